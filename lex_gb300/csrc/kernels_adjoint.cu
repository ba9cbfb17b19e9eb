// kernels_adjoint.cu - vector-Jacobian products (reverse mode) of the big-step operators.
//
// Every kernel is a gather: a thread owns one output adjoint value and sums the contributions
// of the forward outputs that depend on it, so there are no atomics and the results do not
// depend on scheduling.  The forward operators and their reference counterparts:
//
//   acoustic sub-step        one_step_integration.py:519-556 (k_acoustic_vec)
//   WENO flux divergence     advection.py:9-149, fluxes :305-1281 (k_weno_scalars/momentum)
//   mass divergence          advection.py:200-226 (k_div_trho)
//   theta_rho, buoyancy      one_step_integration.py:269, pressure_equations.py:162-172
//   Coriolis                 pressure_gradient_coriolis.py:80-113
//
// WENO adjoint: for each direction a face kernel evaluates, for every flux of the five advected
// fields (theta, qv, u, v, w), the flux adjoint Fbar = (cbar(right) - cbar(left)) / dx, the
// reconstruction W and its derivatives with respect to its stencil, and stores
// Fbar * m * dW/ds as six slots (the cells p-3 .. p+2 of the flux between p-1 and p) plus the
// mass-flux adjoint Fbar * W.  A gather kernel then adds, for every point, the six slots that
// name it and the mass-flux adjoints of the fluxes whose mass flux it enters.
#include "lexgb_adjoint.cuh"
#include "smag_ops.cuh"

namespace lexgb {

namespace {

constexpr int AB = 256;
#define LD(p, idx) __ldg((p) + (idx))

constexpr float kHalfCp = (float)(0.5 * kCp);
constexpr float kRdCvA = (float)(kRd / kCv);

__device__ __forceinline__ int wrapx(int i, int n) { return i < 0 ? i + n : (i >= n ? i - n : i); }

// ---------------------------------------------------------------------------------------------
// reconstruction derivatives
// ---------------------------------------------------------------------------------------------
// W = weno5(a..e) (same formulas as weno5 in lexgb_internal.cuh) and dW/d(a..e) into g[0..4].
__device__ __forceinline__ float weno5_grad(float a, float b, float c, float d, float e, float eps, float* g) {
  const float t1 = a - 2.f * b + c, t2 = a - 4.f * b + 3.f * c;
  const float t3 = b - 2.f * c + d, t4 = b - d;
  const float t5 = c - 2.f * d + e, t6 = 3.f * c - 4.f * d + e;
  const float b1 = (13.f / 12.f) * t1 * t1 + 0.25f * t2 * t2;
  const float b2 = (13.f / 12.f) * t3 * t3 + 0.25f * t4 * t4;
  const float b3 = (13.f / 12.f) * t5 * t5 + 0.25f * t6 * t6;
  const float dd = b1 - b3, tau = fabsf(dd), sg = dd >= 0.f ? 1.f : -1.f;
  // one approximate reciprocal per denominator (the forward divides with div_approx)
  const float i1 = rcp_approx(b1 + eps), i2 = rcp_approx(b2 + eps), i3 = rcp_approx(b3 + eps);
  const float q1r = tau * i1, q2r = tau * i2, q3r = tau * i3;
  const float r1 = fminf(kRatioCap, q1r), r2 = fminf(kRatioCap, q2r), r3 = fminf(kRatioCap, q3r);
  const float w1 = 0.1f * (1.f + r1 * r1), w2 = 0.6f * (1.f + r2 * r2), w3 = 0.3f * (1.f + r3 * r3);
  const float q1 = (2.f / 6.f) * a + (-7.f / 6.f) * b + (11.f / 6.f) * c;
  const float q2 = (-1.f / 6.f) * b + (5.f / 6.f) * c + (2.f / 6.f) * d;
  const float q3 = (2.f / 6.f) * c + (5.f / 6.f) * d + (-1.f / 6.f) * e;
  const float iS = rcp_approx(w1 + w2 + w3);
  const float W = (w1 * q1 + w2 * q2 + w3 * q3) * iS;
  // reverse
  const float qb1 = w1 * iS, qb2 = w2 * iS, qb3 = w3 * iS;
  const float wb1 = (q1 - W) * iS, wb2 = (q2 - W) * iS, wb3 = (q3 - W) * iS;
  const float rb1 = q1r < kRatioCap ? wb1 * 0.2f * r1 : 0.f;
  const float rb2 = q2r < kRatioCap ? wb2 * 1.2f * r2 : 0.f;
  const float rb3 = q3r < kRatioCap ? wb3 * 0.6f * r3 : 0.f;
  const float taub = rb1 * i1 + rb2 * i2 + rb3 * i3;
  const float bb1 = -rb1 * r1 * i1 + taub * sg;
  const float bb2 = -rb2 * r2 * i2;
  const float bb3 = -rb3 * r3 * i3 - taub * sg;
  const float tb1 = bb1 * (13.f / 6.f) * t1, tb2 = bb1 * 0.5f * t2;
  const float tb3 = bb2 * (13.f / 6.f) * t3, tb4 = bb2 * 0.5f * t4;
  const float tb5 = bb3 * (13.f / 6.f) * t5, tb6 = bb3 * 0.5f * t6;
  g[0] = tb1 + tb2 + (2.f / 6.f) * qb1;
  g[1] = -2.f * tb1 - 4.f * tb2 + tb3 + tb4 + (-7.f / 6.f) * qb1 + (-1.f / 6.f) * qb2;
  g[2] = tb1 + 3.f * tb2 - 2.f * tb3 + tb5 + 3.f * tb6 + (11.f / 6.f) * qb1 + (5.f / 6.f) * qb2 + (2.f / 6.f) * qb3;
  g[3] = tb3 - tb4 - 2.f * tb5 - 4.f * tb6 + (2.f / 6.f) * qb2 + (5.f / 6.f) * qb3;
  g[4] = tb5 + tb6 + (-1.f / 6.f) * qb3;
  return W;
}

// W = weno3(a, b, c) and dW/d(a, b, c) into g[0..2].
__device__ __forceinline__ float weno3_grad(float a, float b, float c, float eps, float* g) {
  const float dab = a - b, dbc = b - c;
  const float b1 = dab * dab, b2 = dbc * dbc;
  const float dd = b1 - b2, tau = fabsf(dd), sg = dd >= 0.f ? 1.f : -1.f;
  const float i1 = rcp_approx(b1 + eps), i2 = rcp_approx(b2 + eps);
  const float q1r = tau * i1, q2r = tau * i2;
  const float r1 = fminf(kRatioCap, q1r), r2 = fminf(kRatioCap, q2r);
  const float w1 = (1.f / 3.f) * (1.f + r1 * r1), w2 = (2.f / 3.f) * (1.f + r2 * r2);
  const float q1 = -0.5f * a + 1.5f * b, q2 = 0.5f * b + 0.5f * c;
  const float iS = rcp_approx(w1 + w2);
  const float W = (w1 * q1 + w2 * q2) * iS;
  const float qb1 = w1 * iS, qb2 = w2 * iS;
  const float wb1 = (q1 - W) * iS, wb2 = (q2 - W) * iS;
  const float rb1 = q1r < kRatioCap ? wb1 * (2.f / 3.f) * r1 : 0.f;
  const float rb2 = q2r < kRatioCap ? wb2 * (4.f / 3.f) * r2 : 0.f;
  const float taub = rb1 * i1 + rb2 * i2;
  const float bb1 = -rb1 * r1 * i1 + taub * sg;
  const float bb2 = -rb2 * r2 * i2 - taub * sg;
  g[0] = bb1 * 2.f * dab - 0.5f * qb1;
  g[1] = -bb1 * 2.f * dab + bb2 * 2.f * dbc + 1.5f * qb1 + 0.5f * qb2;
  g[2] = -bb2 * 2.f * dbc + 0.5f * qb2;
  return W;
}

// Lateral face between s[2] and s[3] of s[0..5] (cells p-3 .. p+2): W and dW/ds into g[0..5].
__device__ __forceinline__ float lateral_grad(float m, const float* s, float eps, float* g) {
  float h[5];
  for (int q = 0; q < 6; ++q) g[q] = 0.f;
  if (m >= 0.f) {
    const float W = weno5_grad(s[0], s[1], s[2], s[3], s[4], eps, h);
    for (int q = 0; q < 5; ++q) g[q] = h[q];
    return W;
  }
  const float W = weno5_grad(s[5], s[4], s[3], s[2], s[1], eps, h);
  for (int q = 0; q < 5; ++q) g[5 - q] = h[q];
  return W;
}

// Vertical face H of an n-entry column (between entries H-1 and H), s[0..5] = entries H-3 .. H+2
// (entries outside 0..n-1 are never used); rules of vflux6 in kernels_weno.cu.
__device__ __forceinline__ float vertical_grad(float m, const float* s, int H, int n, float eps, float* g) {
  float h[5];
  for (int q = 0; q < 6; ++q) g[q] = 0.f;
  if (H <= 0 || H >= n) return 0.f;
  const bool up = m >= 0.f;
  if (H >= 3 && H <= n - 3) return lateral_grad(m, s, eps, g);
  if (up) {
    if (H == 1) {
      g[2] = 0.5f;
      g[3] = 0.5f;
      return 0.5f * (s[2] + s[3]);
    }
    if (H == 2 || H == n - 1) {
      const float W = weno3_grad(s[1], s[2], s[3], eps, h);
      g[1] = h[0]; g[2] = h[1]; g[3] = h[2];
      return W;
    }
    const float W = weno5_grad(s[0], s[1], s[2], s[3], s[4], eps, h);  // H == n-2
    for (int q = 0; q < 5; ++q) g[q] = h[q];
    return W;
  }
  if (H == n - 1) {
    g[3] = 0.5f;
    g[2] = 0.5f;
    return 0.5f * (s[3] + s[2]);
  }
  if (H == 1 || H == n - 2) {
    const float W = weno3_grad(s[4], s[3], s[2], eps, h);
    g[4] = h[0]; g[3] = h[1]; g[2] = h[2];
    return W;
  }
  const float W = weno5_grad(s[5], s[4], s[3], s[2], s[1], eps, h);  // H == 2
  for (int q = 0; q < 5; ++q) g[5 - q] = h[q];
  return W;
}

// ---------------------------------------------------------------------------------------------
// acoustic sub-step
// ---------------------------------------------------------------------------------------------
// Values one cell's reverse sub-step reads; neighbour index 0 cell, 1 west, 2 east, 3 south,
// 4 north, 5 below, 6 above.
struct AcNbr {
  float A[7];    // kDivDamp * dtau * adjoint of the output pi'
  float s[7];    // pi'_s
  float p[7];    // input pi'
  float t[7];    // theta_rho
  float unb_w, unb_e, vnb_s, vnb_n, wnb_b, wnb_t;  // adjoints of the output winds on the six faces
  float un_w, un_e, vn_s, vn_n, wn_b, wn_t;        // output winds on the six faces
};
struct AcCol {  // column constants of level k (rho* and their correctly rounded reciprocals *i)
  float pi0m, pi0, pi0p, rhom, rho, rhop, rhomi, rhoi, rhopi, rfb, rft, dzb, dzt;
  bool hb, ht;
};
struct AcOut {
  float ub, vb, wb, pb, tb, sb;
};

__device__ __forceinline__ AcOut acoustic_vjp_cell(const AcNbr& n, const AcCol& k, float pnb0, float rdx, float rdy,
                                                   float rdz, float dtau) {
  const float* A = n.A;
  const float* s = n.s;
  auto divb = [&](int q, float pi0) { return -A[q] * kRdCvA * (pi0 + s[q]); };
  const float D0 = divb(0, k.pi0), DW = divb(1, k.pi0), DE = divb(2, k.pi0), DS = divb(3, k.pi0), DN = divb(4, k.pi0);
  const float DB = k.hb ? divb(5, k.pi0m) : 0.f, DT = k.ht ? divb(6, k.pi0p) : 0.f;
  const float Gw = (s[0] - s[1]) * rdx, Ge = (s[2] - s[0]) * rdx, Gs = (s[0] - s[3]) * rdy, Gn = (s[4] - s[0]) * rdy;
  const float Uw = n.unb_w + (DW - D0) * rdx - 0.5f * Gw * (A[0] + A[1]);
  const float Ue = n.unb_e + (D0 - DE) * rdx - 0.5f * Ge * (A[2] + A[0]);
  const float Vs = n.vnb_s + (DS - D0) * rdy - 0.5f * Gs * (A[0] + A[3]);
  const float Vn = n.vnb_n + (D0 - DN) * rdy - 0.5f * Gn * (A[4] + A[0]);
  float Wb = 0.f, Wt = 0.f;
  if (k.hb) {
    const float Z = k.dzb + (s[0] - s[5]) * rdz;
    Wb = n.wnb_b + (DB - D0) * rdz - 0.5f * Z * k.rfb * (A[0] * k.rhoi + A[5] * k.rhomi);
  }
  if (k.ht) {
    const float Z = k.dzt + (s[6] - s[0]) * rdz;
    Wt = n.wnb_t + (D0 - DT) * rdz - 0.5f * Z * k.rft * (A[6] * k.rhopi + A[0] * k.rhoi);
  }
  AcOut o;
  o.ub = Uw;
  o.vb = Vs;
  o.wb = Wb;
  // pressure-gradient terms of the input pi' and theta_rho
  const float c0 = -kHalfCp * dtau;
  const float* p = n.p;
  const float* t = n.t;
  float pb = pnb0, tb = 0.f;
  pb += Uw * c0 * (t[0] + t[1]) * rdx - Ue * c0 * (t[2] + t[0]) * rdx;
  tb += Uw * c0 * (p[0] - p[1]) * rdx + Ue * c0 * (p[2] - p[0]) * rdx;
  pb += Vs * c0 * (t[0] + t[3]) * rdy - Vn * c0 * (t[4] + t[0]) * rdy;
  tb += Vs * c0 * (p[0] - p[3]) * rdy + Vn * c0 * (p[4] - p[0]) * rdy;
  if (k.hb) {
    pb += Wb * c0 * (t[0] + t[5]) * rdz;
    tb += Wb * c0 * (p[0] - p[5]) * rdz;
  }
  if (k.ht) {
    pb -= Wt * c0 * (t[6] + t[0]) * rdz;
    tb += Wt * c0 * (p[6] - p[0]) * rdz;
  }
  o.pb = pb;
  o.tb = tb;
  // pi'_s: the divergence factor and advection_pi of this cell and its six neighbours
  const float uw = n.un_w, ue = n.un_e, vs = n.vn_s, vn = n.vn_n;
  const float wbn = k.hb ? n.wn_b : 0.f, wtn = k.ht ? n.wn_t : 0.f;
  const float div = (ue - uw) * rdx + (vn - vs) * rdy + (wtn - wbn) * rdz;
  const float dap = -(0.5f * (-ue * rdx + uw * rdx) + 0.5f * (-vn * rdy + vs * rdy) +
                      ((k.hb ? 0.5f * k.rfb * wbn * rdz : 0.f) - (k.ht ? 0.5f * k.rft * wtn * rdz : 0.f)) * k.rhoi);
  float sb = A[0] * (-kRdCvA * div + dap);
  sb += A[2] * 0.5f * ue * rdx - A[1] * 0.5f * uw * rdx;
  sb += A[4] * 0.5f * vn * rdy - A[3] * 0.5f * vs * rdy;
  if (k.ht) sb += A[6] * 0.5f * k.rft * wtn * rdz * k.rhopi;
  if (k.hb) sb -= A[5] * 0.5f * k.rfb * wbn * rdz * k.rhomi;
  o.sb = sb;
  return o;
}

__device__ __forceinline__ AcCol acoustic_col(const Cols& c, int k, int nz) {
  AcCol q;
  q.hb = k > 0;
  q.ht = k + 1 < nz;
  q.pi0 = c.pi0[k];
  q.rho = c.rho[k];
  q.rhoi = c.rho_inv[k];
  q.pi0m = q.hb ? c.pi0[k - 1] : 0.f;
  q.rhom = q.hb ? c.rho[k - 1] : 1.f;
  q.rhomi = q.hb ? c.rho_inv[k - 1] : 1.f;
  q.pi0p = q.ht ? c.pi0[k + 1] : 0.f;
  q.rhop = q.ht ? c.rho[k + 1] : 1.f;
  q.rhopi = q.ht ? c.rho_inv[k + 1] : 1.f;
  q.rfb = c.rho_face[k];
  q.rft = c.rho_face[k + 1];
  q.dzb = c.dpi0dz[k];
  q.dzt = c.dpi0dz[k + 1];
  return q;
}

// one thread per cell (any nx)
__global__ void __launch_bounds__(AB) k_acoustic_vjp(Dims d, Phys ph, Cols c, AcousticVjpArgs a, float dtau) {
  const long long t = (long long)blockIdx.x * AB + threadIdx.x;
  const int nx = d.nx, ny = d.ny, nz = d.nz, plane = d.plane();
  if (t >= d.cells()) return;
  const int i = (int)(t % nx), j = (int)((t / nx) % ny), k = (int)(t / plane);
  const int id = (int)t, row = k * plane + j * nx;
  const AcCol col = acoustic_col(c, k, nz);
  int q[7];
  q[0] = id;
  q[1] = row + wrapx(i - 1, nx);
  q[2] = row + wrapx(i + 1, nx);
  q[3] = k * plane + wrapx(j - 1, ny) * nx + i;
  q[4] = k * plane + wrapx(j + 1, ny) * nx + i;
  q[5] = col.hb ? id - plane : id;
  q[6] = col.ht ? id + plane : id;
  const float K = kDivDamp * dtau;
  AcNbr n;
#pragma unroll
  for (int m = 0; m < 7; ++m) {
    const bool ok = (m < 5) || (m == 5 ? col.hb : col.ht);
    n.A[m] = ok ? K * LD(a.pnb, q[m]) : 0.f;
    n.s[m] = ok ? LD(a.ps, q[m]) : 0.f;
    n.p[m] = ok ? LD(a.p, q[m]) : 0.f;
    n.t[m] = ok ? LD(a.trho, q[m]) : 0.f;
  }
  n.unb_w = LD(a.unb, id); n.unb_e = LD(a.unb, q[2]);
  n.vnb_s = LD(a.vnb, id); n.vnb_n = LD(a.vnb, q[4]);
  n.wnb_b = LD(a.wnb, id); n.wnb_t = LD(a.wnb, id + plane);
  n.un_w = LD(a.un, id); n.un_e = LD(a.un, q[2]);
  n.vn_s = LD(a.vn, id); n.vn_n = LD(a.vn, q[4]);
  n.wn_b = LD(a.wn, id); n.wn_t = LD(a.wn, id + plane);
  const AcOut o = acoustic_vjp_cell(n, col, LD(a.pnb, id), ph.rdx, ph.rdy, ph.rdz, dtau);
  a.ub[id] = o.ub;
  a.vb[id] = o.vb;
  a.wb[id] = o.wb;
  if (k == nz - 1) a.wb[id + plane] = 0.f;
  a.pb[id] = o.pb;
  a.Rub[id] += o.ub * dtau;
  a.Rvb[id] += o.vb * dtau;
  if (col.hb) a.Rwb[id] += o.wb * dtau;
  a.trhob[id] += o.tb;
  a.psb[id] += o.sb;
}

// V consecutive x cells per thread (V = 2 or 4) with V-wide row loads (nx % V == 0), as
// k_acoustic_vec
#ifndef ACOUSTIC_VJP_VEC
#define ACOUSTIC_VJP_VEC 4
#endif
template <int V>
struct VecF;
template <>
struct VecF<4> {
  typedef float4 T;
};
template <>
struct VecF<2> {
  typedef float2 T;
};
template <int V>
__device__ __forceinline__ void ldvec(const float* p, int i, float (&o)[V]) {
  typedef typename VecF<V>::T T;
  const T t = __ldg(reinterpret_cast<const T*>(p + i));
  const float* f = reinterpret_cast<const float*>(&t);
#pragma unroll
  for (int l = 0; l < V; ++l) o[l] = f[l];
}
template <int V>
__device__ __forceinline__ void stvec(float* p, int i, const float (&v)[V]) {
  typedef typename VecF<V>::T T;
  T t;
  float* f = reinterpret_cast<float*>(&t);
#pragma unroll
  for (int l = 0; l < V; ++l) f[l] = v[l];
  *reinterpret_cast<T*>(p + i) = t;
}
template <int V>
__device__ __forceinline__ void accvec(float* p, int i, const float (&v)[V], float s) {
  typedef typename VecF<V>::T T;
  T t = *reinterpret_cast<T*>(p + i);
  float* f = reinterpret_cast<float*>(&t);
#pragma unroll
  for (int l = 0; l < V; ++l) f[l] += v[l] * s;
  *reinterpret_cast<T*>(p + i) = t;
}

template <int V>
__global__ void __launch_bounds__(64) k_acoustic_vjpv(Dims d, Phys ph, Cols c, AcousticVjpArgs a, float dtau) {
  const int nq = d.nx / V;
  const int qx = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  const int k = blockIdx.z;
  if (qx >= nq || j >= d.ny) return;
  const int nx = d.nx, ny = d.ny, nz = d.nz, plane = d.plane();
  const int i0 = V * qx;
  const int r0 = k * plane + j * nx, rs = k * plane + wrapx(j - 1, ny) * nx, rn = k * plane + wrapx(j + 1, ny) * nx;
  const int iw = wrapx(i0 - 1, nx), ie = wrapx(i0 + V, nx);
  const AcCol col = acoustic_col(c, k, nz);
  const int rb = col.hb ? r0 - plane : r0, rt = col.ht ? r0 + plane : r0;
  const float K = kDivDamp * dtau;
  // rows: 0 centre, 1 south, 2 north, 3 below, 4 above
  const int rows[5] = {r0, rs, rn, rb, rt};
  float PN[5][V], PS[5][V], PP[5][V], TT[5][V];
#pragma unroll
  for (int r = 0; r < 5; ++r) {
    ldvec<V>(a.pnb, rows[r] + i0, PN[r]);
    ldvec<V>(a.ps, rows[r] + i0, PS[r]);
    ldvec<V>(a.p, rows[r] + i0, PP[r]);
    ldvec<V>(a.trho, rows[r] + i0, TT[r]);
  }
  const float pnW = LD(a.pnb, r0 + iw), pnE = LD(a.pnb, r0 + ie);
  const float psW = LD(a.ps, r0 + iw), psE = LD(a.ps, r0 + ie);
  const float ppW = LD(a.p, r0 + iw), ppE = LD(a.p, r0 + ie);
  const float ttW = LD(a.trho, r0 + iw), ttE = LD(a.trho, r0 + ie);
  float UNB[V], VNB[V], VNBn[V], WNB[V], WNBt[V], UN[V], VN[V], VNn[V], WN[V], WNt[V];
  ldvec<V>(a.unb, r0 + i0, UNB);
  ldvec<V>(a.vnb, r0 + i0, VNB);
  ldvec<V>(a.vnb, rn + i0, VNBn);
  ldvec<V>(a.wnb, r0 + i0, WNB);
  ldvec<V>(a.wnb, r0 + plane + i0, WNBt);
  ldvec<V>(a.un, r0 + i0, UN);
  ldvec<V>(a.vn, r0 + i0, VN);
  ldvec<V>(a.vn, rn + i0, VNn);
  ldvec<V>(a.wn, r0 + i0, WN);
  ldvec<V>(a.wn, r0 + plane + i0, WNt);
  const float unbE = LD(a.unb, r0 + ie), unE = LD(a.un, r0 + ie);
  float ob[V], vb[V], wb[V], pb[V], tb[V], sb[V];
#pragma unroll
  for (int l = 0; l < V; ++l) {
    AcNbr n;
    // x neighbours inside the vector or the scalar ends
    const float pnw = l == 0 ? pnW : PN[0][l - 1], pne = l == V - 1 ? pnE : PN[0][l + 1];
    const float psw = l == 0 ? psW : PS[0][l - 1], pse = l == V - 1 ? psE : PS[0][l + 1];
    const float ppw = l == 0 ? ppW : PP[0][l - 1], ppe = l == V - 1 ? ppE : PP[0][l + 1];
    const float ttw = l == 0 ? ttW : TT[0][l - 1], tte = l == V - 1 ? ttE : TT[0][l + 1];
    n.A[0] = K * PN[0][l]; n.A[1] = K * pnw; n.A[2] = K * pne;
    n.A[3] = K * PN[1][l]; n.A[4] = K * PN[2][l];
    n.A[5] = col.hb ? K * PN[3][l] : 0.f; n.A[6] = col.ht ? K * PN[4][l] : 0.f;
    n.s[0] = PS[0][l]; n.s[1] = psw; n.s[2] = pse; n.s[3] = PS[1][l]; n.s[4] = PS[2][l];
    n.s[5] = PS[3][l]; n.s[6] = PS[4][l];
    n.p[0] = PP[0][l]; n.p[1] = ppw; n.p[2] = ppe; n.p[3] = PP[1][l]; n.p[4] = PP[2][l];
    n.p[5] = PP[3][l]; n.p[6] = PP[4][l];
    n.t[0] = TT[0][l]; n.t[1] = ttw; n.t[2] = tte; n.t[3] = TT[1][l]; n.t[4] = TT[2][l];
    n.t[5] = TT[3][l]; n.t[6] = TT[4][l];
    n.unb_w = UNB[l]; n.unb_e = l == V - 1 ? unbE : UNB[l + 1];
    n.vnb_s = VNB[l]; n.vnb_n = VNBn[l];
    n.wnb_b = WNB[l]; n.wnb_t = WNBt[l];
    n.un_w = UN[l]; n.un_e = l == V - 1 ? unE : UN[l + 1];
    n.vn_s = VN[l]; n.vn_n = VNn[l];
    n.wn_b = WN[l]; n.wn_t = WNt[l];
    const AcOut o = acoustic_vjp_cell(n, col, PN[0][l], ph.rdx, ph.rdy, ph.rdz, dtau);
    ob[l] = o.ub; vb[l] = o.vb; wb[l] = o.wb; pb[l] = o.pb; tb[l] = o.tb; sb[l] = o.sb;
  }
  stvec<V>(a.ub, r0 + i0, ob);
  stvec<V>(a.vb, r0 + i0, vb);
  stvec<V>(a.wb, r0 + i0, wb);
  stvec<V>(a.pb, r0 + i0, pb);
  if (k == nz - 1) {
    float z[V];
#pragma unroll
    for (int l = 0; l < V; ++l) z[l] = 0.f;
    stvec<V>(a.wb, r0 + plane + i0, z);
  }
  accvec<V>(a.Rub, r0 + i0, ob, dtau);
  accvec<V>(a.Rvb, r0 + i0, vb, dtau);
  if (col.hb) accvec<V>(a.Rwb, r0 + i0, wb, dtau);
  accvec<V>(a.trhob, r0 + i0, tb, 1.f);
  accvec<V>(a.psb, r0 + i0, sb, 1.f);
}

// ---------------------------------------------------------------------------------------------
// pointwise part of a stage's reverse pass (after the acoustic loop):
//   cbar of the five advected fields, the phi*div terms, Coriolis, buoyancy, theta_rho,
//   pi'_s, SGS adjoints and the identity paths to xi0
// ---------------------------------------------------------------------------------------------
__global__ void __launch_bounds__(AB) k_stage_pointwise_vjp(Dims d, Phys ph, Cols c, StageVjpArgs a) {
  const long long t = (long long)blockIdx.x * AB + threadIdx.x;
  const int nx = d.nx, ny = d.ny, nz = d.nz, plane = d.plane();
  if (t >= d.faces()) return;
  const int i = (int)(t % nx), j = (int)((t / nx) % ny), k = (int)(t / plane);
  const int id = (int)t;
  const int im = wrapx(i - 1, nx), ip = wrapx(i + 1, nx), jm = wrapx(j - 1, ny), jp = wrapx(j + 1, ny);
  const int row = k * plane;
  // ---- w point (face k): cbar_w, the w*div term, buoyancy is gathered at cells below
  {
    float cw = 0.f, wb = 0.f;
    const float Rw = LD(a.Rwb, id);
    if (k >= 1 && k < nz) {
      const float deni = c.rho_w_inv[k];   // 1 / (0.5 (rho0(k-1) + rho0(k)))
      cw = Rw * deni;
      wb = Rw * 0.5f * (LD(a.div, id - plane) + LD(a.div, id)) * deni;
    }
    a.cb[2][id] = cw;
    a.xsb.w[id] += wb;
    a.x0b.w[id] += LD(a.acb[2], id);   // the acoustic loop starts from the big step's input winds and pi'
    if (a.sgsb_w && k >= 1 && k < nz) a.sgsb_w[id] += Rw;
  }
  if (k >= nz) return;
  a.x0b.u[id] += LD(a.acb[0], id);
  a.x0b.v[id] += LD(a.acb[1], id);
  a.x0b.p[id] += LD(a.acb[3], id);
  const float ri = c.rho_inv[k];   // products with the correctly rounded 1 / rho0 instead of divisions
  // ---- scalars
  const float Tb = LD(a.Tnb, id), Qb = LD(a.qnb, id);
  const float cT = a.dts * Tb * ri, cQ = a.dts * Qb * ri;
  a.cb[3][id] = cT;
  a.cb[4][id] = cQ;
  const float dv = LD(a.div, id);
  const float T = LD(a.xs.T, id), q = LD(a.xs.q, id);
  float dvb = cT * T + cQ * q;
  float Tsb = cT * dv, qsb = cQ * dv;
  a.x0b.T[id] += Tb;
  a.x0b.q[id] += Qb;
  if (a.sgsb_T) {
    a.sgsb_T[id] += a.dts * Tb;
    a.sgsb_q[id] += a.dts * Qb;
  }
  // ---- u, v points
  const float Ru = LD(a.Rub, id), Rv = LD(a.Rvb, id);
  a.cb[0][id] = Ru * ri;
  a.cb[1][id] = Rv * ri;
  float ub = Ru * 0.5f * (LD(a.div, row + j * nx + im) + dv) * ri;
  float vb = Rv * 0.5f * (LD(a.div, row + jm * nx + i) + dv) * ri;
  if (a.sgsb_u) {
    a.sgsb_u[id] += Ru;
    a.sgsb_v[id] += Rv;
  }
  // divergence adjoint of this cell from the phi*div terms of its u, v, w points
  dvb += 0.5f * ri * (Ru * LD(a.xs.u, id) + LD(a.Rub, row + j * nx + ip) * LD(a.xs.u, row + j * nx + ip));
  dvb += 0.5f * ri * (Rv * LD(a.xs.v, id) + LD(a.Rvb, row + jp * nx + i) * LD(a.xs.v, row + jp * nx + i));
  if (k >= 1) dvb += 0.5f * LD(a.Rwb, id) * LD(a.xs.w, id) * c.rho_w_inv[k];
  if (k + 1 < nz) dvb += 0.5f * LD(a.Rwb, id + plane) * LD(a.xs.w, id + plane) * c.rho_w_inv[k + 1];
  // Coriolis: R_u += f v4, R_v -= f u4 (both cor_opt 1 and 2 are linear in the winds)
  if (ph.cor_opt) {
    const float f4 = 0.25f * ph.f_cor;
    vb += f4 * (Ru + LD(a.Rub, row + j * nx + ip) + LD(a.Rub, row + jm * nx + i) + LD(a.Rub, row + jm * nx + ip));
    ub -= f4 * (Rv + LD(a.Rvb, row + jp * nx + i) + LD(a.Rvb, row + j * nx + im) + LD(a.Rvb, row + jp * nx + im));
  }
  a.xsb.u[id] += ub;
  a.xsb.v[id] += vb;
  a.divb[id] = dvb;
  // buoyancy b(k) enters b8w on faces k and k+1 (the end faces' extrapolations meet a zero R_w
  // adjoint: the acoustic sub-step pins w there)
  {
    const float bb = 0.5f * ((k >= 1 ? LD(a.Rwb, id) : 0.f) + (k + 1 < nz ? LD(a.Rwb, id + plane) : 0.f));
    const float th0 = c.theta0[k], q0 = c.qv0[k], tr0 = c.trho0[k];
    const float reps = (float)kReps;
    const float num = th0 * (float)(kReps - 1.0) * (q - q0) + (T - c.d0[k]) * (1.f + reps * q) * (1.f + q0);
    const float den = (1.f + q) * (1.f + q0);
    const float g = (float)kG / tr0;
    Tsb += bb * g * (1.f + reps * q) * (1.f + q0) / den;
    const float dnum = th0 * (float)(kReps - 1.0) + (T - c.d0[k]) * reps * (1.f + q0);
    qsb += bb * g * (dnum * den - num * (1.f + q0)) / (den * den);
  }
  // theta_rho = (theta_ref + T)(1 + reps q)/(1 + q)
  {
    const float trb = LD(a.trhob, id);
    const float reps = (float)kReps;
    Tsb += trb * (1.f + reps * q) / (1.f + q);
    qsb += trb * (ph.theta_ref + T) * (reps - 1.f) / ((1.f + q) * (1.f + q));
  }
  a.xsb.T[id] += Tsb;
  a.xsb.q[id] += qsb;
  a.xsb.p[id] += LD(a.psb, id);
}

// mass divergence: xsb winds += div^T(divb)
// and, with x0b (the first stage, whose input is the big step's input): x0b += xsb, all six fields
__global__ void __launch_bounds__(AB) k_massdiv_vjp(Dims d, Phys ph, Cols c, const float* __restrict__ divb, State xsb,
                                                    State x0b) {
  const long long t = (long long)blockIdx.x * AB + threadIdx.x;
  const int nx = d.nx, ny = d.ny, nz = d.nz, plane = d.plane();
  if (t >= d.faces()) return;
  const int i = (int)(t % nx), j = (int)((t / nx) % ny), k = (int)(t / plane);
  const int id = (int)t;
  if (k >= 1 && k < nz) xsb.w[id] += c.rho_face0[k] * (LD(divb, id - plane) - LD(divb, id)) * ph.rdz;
  if (x0b.w) x0b.w[id] += xsb.w[id];
  if (k >= nz) return;
  const float r = c.rho[k];
  const int row = k * plane;
  xsb.u[id] += r * (LD(divb, row + j * nx + wrapx(i - 1, nx)) - LD(divb, id)) * ph.rdx;
  xsb.v[id] += r * (LD(divb, row + wrapx(j - 1, ny) * nx + i) - LD(divb, id)) * ph.rdy;
  if (x0b.u) {
    x0b.u[id] += xsb.u[id];
    x0b.v[id] += xsb.v[id];
    x0b.T[id] += xsb.T[id];
    x0b.q[id] += xsb.q[id];
    x0b.p[id] += xsb.p[id];
  }
}

// ---------------------------------------------------------------------------------------------
// WENO advection adjoint, one direction
// ---------------------------------------------------------------------------------------------
// point p of field f along direction D: neighbour at offset o (wrapped / or -1 outside the column)
template <int D>
__device__ __forceinline__ int along(const Dims& d, int i, int j, int k, int o, int n) {
  if (D == 0) return (k * d.ny + j) * d.nx + wrapx(i + o, d.nx);
  if (D == 1) return (k * d.ny + wrapx(j + o, d.ny)) * d.nx + i;
  const int kk = k + o;
  return (kk < 0 || kk >= n) ? -1 : (kk * d.ny + j) * d.nx + i;
}

// fields: 0 u, 1 v, 2 w, 3 theta, 4 qv
template <int D>
__global__ void __launch_bounds__(AB) k_adv_face_vjp(Dims d, Phys ph, Cols c, AdvVjpArgs a) {
  const long long t = (long long)blockIdx.x * AB + threadIdx.x;
  const int nx = d.nx, ny = d.ny, nz = d.nz, plane = d.plane();
  if (t >= d.faces()) return;
  const int i = (int)(t % nx), j = (int)((t / nx) % ny), k = (int)(t / plane);
  const int id = (int)t;
  const float rd = D == 0 ? ph.rdx : (D == 1 ? ph.rdy : ph.rdz);
  const int im = wrapx(i - 1, nx), jm = wrapx(j - 1, ny);
  float mbar_s = 0.f;
  for (int f = 0; f < 5; ++f) {
    const int n = f == 2 ? nz + 1 : nz;  // points in the field's column
    const float* phi = a.phi[f];
    float slots[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    float mbar = 0.f;
    bool valid;
    if (D < 2)
      valid = f == 2 ? (k >= 1 && k < nz) : (k < nz);
    else
      valid = k >= 1 && k < n;  // face H = k between column entries k-1 and k
    if (valid) {
      // mass flux
      float m;
      const float r = k < nz ? c.rho[k] : 0.f, rm = k >= 1 ? c.rho[k - 1] : 0.f;
      if (D == 0) {
        const float* u = a.xs.u;
        if (f == 0) m = 0.5f * (LD(u, (k * ny + j) * nx + im) + LD(u, id)) * r;
        else if (f == 1) m = 0.5f * (r * LD(u, (k * ny + jm) * nx + i) + r * LD(u, id));
        else if (f == 2) m = 0.5f * (rm * LD(u, id - plane) + r * LD(u, id));
        else m = r * LD(u, id);
      } else if (D == 1) {
        const float* v = a.xs.v;
        if (f == 0) m = 0.5f * (r * LD(v, (k * ny + j) * nx + im) + r * LD(v, id));
        else if (f == 1) m = 0.5f * (LD(v, (k * ny + jm) * nx + i) + LD(v, id)) * r;
        else if (f == 2) m = 0.5f * (rm * LD(v, id - plane) + r * LD(v, id));
        else m = r * LD(v, id);
      } else {
        const float* w = a.xs.w;
        const float rf = c.rho_face[k];
        if (f == 0) m = 0.5f * (rf * LD(w, (k * ny + j) * nx + im) + rf * LD(w, id));
        else if (f == 1) m = 0.5f * (rf * LD(w, (k * ny + jm) * nx + i) + rf * LD(w, id));
        else if (f == 2) m = 0.5f * (LD(w, id - plane) + LD(w, id)) * rm;
        else m = rf * LD(w, id);
      }
      // flux adjoint: the flux between points p-1 and p leaves p-1 and enters p
      const int pm = along<D>(d, i, j, k, -1, n);
      const float Fb = (LD(a.cb[f], id) - LD(a.cb[f], pm)) * rd;
      float s[6];
      for (int q = 0; q < 6; ++q) {
        const int pq = along<D>(d, i, j, k, q - 3, n);
        s[q] = pq >= 0 ? LD(phi, pq) : 0.f;
      }
      const float eps = f < 3 ? kWepsMom : (f == 3 ? kWepsTheta : kWepsQv);
      float g[6];
      const float W = D < 2 ? lateral_grad(m, s, eps, g) : vertical_grad(m, s, k, n, eps, g);
      for (int q = 0; q < 6; ++q) slots[q] = Fb * m * g[q];
      mbar = Fb * W;
    }
    for (int q = 0; q < 6; ++q) a.P[f][q][id] = slots[q];
    if (f < 3) a.mb[f][id] = mbar;
    else mbar_s += mbar;
  }
  a.mb[3][id] = mbar_s;
}

template <int D>
__global__ void __launch_bounds__(AB) k_adv_gather_vjp(Dims d, Phys ph, Cols c, AdvVjpArgs a) {
  const long long t = (long long)blockIdx.x * AB + threadIdx.x;
  const int nx = d.nx, ny = d.ny, nz = d.nz, plane = d.plane();
  if (t >= d.faces()) return;
  const int i = (int)(t % nx), j = (int)((t / nx) % ny), k = (int)(t / plane);
  const int id = (int)t;
  float* out[5] = {a.xsb.u, a.xsb.v, a.xsb.w, a.xsb.T, a.xsb.q};
  for (int f = 0; f < 5; ++f) {
    const int n = f == 2 ? nz + 1 : nz;
    if (k >= n) continue;
    float acc = 0.f;
    // the flux at point p+3-q names this point in its slot q
    for (int q = 0; q < 6; ++q) {
      const int pf = along<D>(d, i, j, k, 3 - q, nz + 1);  // fluxes exist on face levels 0..nz
      if (pf >= 0) acc += LD(a.P[f][q], pf);
    }
    out[f][id] += acc;
  }
  // mass-flux adjoints into the wind of direction D
  const int ip = wrapx(i + 1, nx), jp = wrapx(j + 1, ny);
  if (D == 0) {
    if (k >= nz) return;
    const float r = c.rho[k];
    const int row = k * plane;
    float ub = r * LD(a.mb[3], id);                                                     // theta, qv
    ub += 0.5f * r * (LD(a.mb[0], id) + LD(a.mb[0], row + j * nx + ip));                // u
    ub += 0.5f * r * (LD(a.mb[1], id) + LD(a.mb[1], row + wrapx(j + 1, ny) * nx + i));  // v (corner)
    ub += 0.5f * r * ((k >= 1 ? LD(a.mb[2], id) : 0.f) + (k + 1 < nz ? LD(a.mb[2], id + plane) : 0.f));  // w
    a.xsb.u[id] += ub;
  } else if (D == 1) {
    if (k >= nz) return;
    const float r = c.rho[k];
    const int row = k * plane;
    float vb = r * LD(a.mb[3], id);
    vb += 0.5f * r * (LD(a.mb[0], id) + LD(a.mb[0], row + j * nx + ip));
    vb += 0.5f * r * (LD(a.mb[1], id) + LD(a.mb[1], row + jp * nx + i));
    vb += 0.5f * r * ((k >= 1 ? LD(a.mb[2], id) : 0.f) + (k + 1 < nz ? LD(a.mb[2], id + plane) : 0.f));
    a.xsb.v[id] += vb;
  } else {
    const int row = k * plane;
    float wb = 0.f;
    if (k >= 1 && k < nz) {
      const float rf = c.rho_face[k];
      wb += rf * LD(a.mb[3], id);
      wb += 0.5f * rf * (LD(a.mb[0], id) + LD(a.mb[0], row + j * nx + ip));
      wb += 0.5f * rf * (LD(a.mb[1], id) + LD(a.mb[1], row + jp * nx + i));
    }
    if (k >= 1) wb += 0.5f * c.rho[k - 1] * LD(a.mb[2], id);
    if (k + 1 <= nz) wb += 0.5f * c.rho[k] * LD(a.mb[2], id + plane);
    a.xsb.w[id] += wb;
  }
}

// ---------------------------------------------------------------------------------------------
// Smagorinsky (turbulence.py:9-111, :298-446) backwards
// ---------------------------------------------------------------------------------------------
// weight of the edge value e13 / e23 on w face f in s13 / s23 of cell level k (without rho):
// corner averages inside, the quadratic end extrapolation in the bottom and top cells
__device__ __forceinline__ float w_edge(int k, int f, int nz) {
  if (k == 0) return f == 1 ? 0.5f * 1.875f : (f == 2 ? 0.5f * -1.25f : (f == 3 ? 0.5f * 0.375f : 0.f));
  if (k == nz - 1) return f == nz - 1 ? 0.5f * 1.875f : (f == nz - 2 ? 0.5f * -1.25f : (f == nz - 3 ? 0.5f * 0.375f : 0.f));
  return (f == k || f == k + 1) ? 0.25f : 0.f;
}
// weight of n2_face(f) in N^2 of cell level k
__device__ __forceinline__ float w_n2(int k, int f, int nz) {
  if (k == 0) return f == 1 ? 1.875f : (f == 2 ? -1.25f : (f == 3 ? 0.375f : 0.f));
  if (k == nz - 1) return f == nz - 1 ? 1.875f : (f == nz - 2 ? -1.25f : (f == nz - 3 ? 0.375f : 0.f));
  return (f == k || f == k + 1) ? 0.5f : 0.f;
}
// the cell levels whose s13 / s23 / N^2 read face f: f-1, f and the two end cells (distinct)
__device__ __forceinline__ int face_cells(int f, int nz, int* ks) {
  int n = 0;
  ks[n++] = f - 1;
  ks[n++] = f;
  if (f - 1 != 0 && f != 0) ks[n++] = 0;
  if (f - 1 != nz - 1 && f != nz - 1) ks[n++] = nz - 1;
  return n;
}

// forward quantities of compute_deformation / compute_nm / compute_k at every cell (as k_smag_a)
__global__ void __launch_bounds__(AB) k_smag_lin(Dims d, Phys ph, Cols c, State s, SmagLin o) {
  using namespace smag;
  const long long t = (long long)blockIdx.x * AB + threadIdx.x;
  if (t >= d.cells()) return;
  const int nx = d.nx, ny = d.ny, nz = d.nz;
  const int i = (int)(t % nx), j = (int)((t / nx) % ny), k = (int)(t / d.plane());
  const int id = (int)t;
  const float r = c.rho[k], ri = c.rho_inv[k];
  const int ip = wrap(i + 1, nx), jp = wrap(j + 1, ny);
  const float s11 = r * (LD(s.u, d.at(ip, j, k)) - LD(s.u, id)) * ph.rdx;
  const float s22 = r * (LD(s.v, d.at(i, jp, k)) - LD(s.v, id)) * ph.rdy;
  const float s33 = r * (LD(s.w, d.at(i, j, k + 1)) - LD(s.w, id)) * ph.rdz;
  const float s12 = r * (0.25f * (e12(d, ph, s, i, j, k) + e12(d, ph, s, i + 1, j + 1, k) + e12(d, ph, s, i, j + 1, k) +
                                  e12(d, ph, s, i + 1, j, k)));
  float s13 = 0.f, s23 = 0.f, n2 = 0.f;
  // faces with nonzero weight: k, k+1 inside, 1..3 / nz-3..nz-1 in the end cells
  const int f0 = k == 0 ? 1 : (k == nz - 1 ? nz - 3 : k), f1 = k == 0 ? 3 : (k == nz - 1 ? nz - 1 : k + 1);
  for (int f = f0; f <= f1; ++f) {
    const float we = w_edge(k, f, nz), wn = w_n2(k, f, nz);
    if (we != 0.f) {
      s13 += we * (e13(d, ph, s, i, j, f) + e13(d, ph, s, i + 1, j, f));
      s23 += we * (e23(d, ph, s, i, j, f) + e23(d, ph, s, i, j + 1, f));
    }
    if (wn != 0.f) n2 += wn * n2_face(d, ph, s, i, j, f);
  }
  s13 *= r;
  s23 *= r;
  const float s2 = (2.f * (s11 * s11 + s22 * s22 + s33 * s33) + 4.f * (s12 * s12 + s13 * s13 + s23 * s23)) * (ri * ri);
  const float s2n2 = s2 - n2 * kInvPrandtl;
  const float km = s2n2 > 0.f ? ph.smag_l2 * sqrtf(s2n2) : 0.f;
  o.s[0][id] = s11; o.s[1][id] = s22; o.s[2][id] = s33; o.s[3][id] = s12; o.s[4][id] = s13; o.s[5][id] = s23;
  o.km[id] = km;
  o.kS[id] = s2n2 > 0.f ? 0.5f * ph.smag_l2 / sqrtf(s2n2) : 0.f;
}

// adjoint of compute_smag: tau_ij, K_h and the direct theta / qv terms of the scalar diffusion
__global__ void __launch_bounds__(AB) k_smag_tau_vjp(Dims d, Phys ph, Cols c, State s, SmagLin l, SmagVjpArgs a) {
  const long long t = (long long)blockIdx.x * AB + threadIdx.x;
  if (t >= d.cells()) return;
  const int nx = d.nx, ny = d.ny, nz = d.nz, plane = d.plane();
  const int i = (int)(t % nx), j = (int)((t / nx) % ny), k = (int)(t / plane);
  const int id = (int)t;
  const int im = wrapx(i - 1, nx), ip = wrapx(i + 1, nx), jm = wrapx(j - 1, ny), jp = wrapx(j + 1, ny);
  const float rdx = ph.rdx, rdy = ph.rdy, rdz = ph.rdz;
  const float r = c.rho[k], ri = c.rho_inv[k];   // ri: the correctly rounded 1 / rho0, multiplied instead of divided
  auto at = [&](int ii, int jj, int kk) { return (kk * ny + jj) * nx + ii; };
  const float* U = a.gu;
  const float* V = a.gv;
  const float* W = a.gw;
  // tau11, tau22, tau33
  a.tb[0][id] = (LD(U, at(ip, j, k)) - LD(U, id)) * rdx * ri;
  a.tb[1][id] = (LD(V, at(i, jp, k)) - LD(V, id)) * rdy * ri;
  float t33 = 0.f;
  if (k >= 1) t33 -= LD(W, id) * rdz * c.rho_wext_inv[k];
  if (k + 1 <= nz - 1) t33 += LD(W, id + plane) * rdz * c.rho_wext_inv[k + 1];
  a.tb[2][id] = t33;
  // tau12 through d12v (sgs_u) and d12u (sgs_v)
  {
    auto d12v = [&](int cc, int jf) {  // adjoint of (t12(cc,jf) - t12(cc,jf-1)) rdy
      const int c1 = wrapx(cc + 1, nx), c0 = wrapx(cc, nx), j0 = wrapx(jf, ny), j1 = wrapx(jf - 1, ny);
      return -0.25f * ri * (LD(U, at(c1, j0, k)) + LD(U, at(c0, j1, k)) + LD(U, at(c1, j1, k)) + LD(U, at(c0, j0, k)));
    };
    auto d12u = [&](int q, int rr) {  // adjoint of (t12(q,rr) - t12(q-1,rr)) rdx
      const int q0 = wrapx(q, nx), q1 = wrapx(q - 1, nx), r0 = wrapx(rr, ny), r1 = wrapx(rr + 1, ny);
      return -0.25f * ri * (LD(V, at(q0, r1, k)) + LD(V, at(q1, r0, k)) + LD(V, at(q0, r0, k)) + LD(V, at(q1, r1, k)));
    };
    a.tb[3][id] = rdy * (d12v(i, j) - d12v(i, j + 1)) + rdx * (d12u(i, j) - d12u(i + 1, j));
  }
  // tau13, tau23: sgs_w (centred lateral differences averaged to faces) and sgs_u / sgs_v
  {
    float t13 = 0.f, t23 = 0.f;
    for (int kf = k; kf <= k + 1; ++kf) {
      if (kf < 1 || kf > nz - 1) continue;
      const float cw = -0.5f * c.rho_wext_inv[kf];
      t13 += cw * (LD(W, at(im, j, kf)) - LD(W, at(ip, j, kf))) / (2.f * ph.dx);
      t23 += cw * (LD(W, at(i, jm, kf)) - LD(W, at(i, jp, kf))) / (2.f * ph.dy);
      // d13s(cc, k') = (to_w0(t13(cc), k'+1) - to_w0(t13(cc), k')) rdz enters sgs_u(cc), sgs_u(cc+1)
      auto d13s = [&](int kk) { return -0.5f * c.rho_inv[kk] * (LD(U, at(ip, j, kk)) + LD(U, at(i, j, kk))); };
      auto d23s = [&](int kk) { return -0.5f * c.rho_inv[kk] * (LD(V, at(i, jp, kk)) + LD(V, at(i, j, kk))); };
      t13 += 0.5f * rdz * (d13s(kf - 1) - d13s(kf));
      t23 += 0.5f * rdz * (d23s(kf - 1) - d23s(kf));
    }
    a.tb[4][id] = t13;
    a.tb[5][id] = t23;
  }
  // scalar diffusion of theta and qv: direct terms and K_h
  {
    const float khc = LD(l.km, id) * kInvPrandtl;
    auto kh = [&](int q) { return LD(l.km, q) * kInvPrandtl; };
    const int nb[4] = {at(im, j, k), at(ip, j, k), at(i, jm, k), at(i, jp, k)};
    float khb = 0.f;
    for (int fld = 0; fld < 2; ++fld) {
      const float* A = fld == 0 ? s.T : s.q;
      const float* G = fld == 0 ? a.gT : a.gq;
      const float a0 = LD(A, id), g0 = LD(G, id);
      float ab = 0.f;
      // x faces i (west) and i+1 (east), y faces j and j+1
      {
        const float fw = (g0 - LD(G, nb[0])) * rdx * ri, fe = (LD(G, nb[1]) - g0) * rdx * ri;
        const float k8w = 0.5f * (khc + kh(nb[0])), k8e = 0.5f * (kh(nb[1]) + khc);
        ab += -r * rdx * (fw * k8w - fe * k8e);
        khb += 0.5f * (fw * (-r * (a0 - LD(A, nb[0])) * rdx) + fe * (-r * (LD(A, nb[1]) - a0) * rdx));
        const float fs = (g0 - LD(G, nb[2])) * rdy * ri, fn = (LD(G, nb[3]) - g0) * rdy * ri;
        const float k8s = 0.5f * (khc + kh(nb[2])), k8n = 0.5f * (kh(nb[3]) + khc);
        ab += -r * rdy * (fs * k8s - fn * k8n);
        khb += 0.5f * (fs * (-r * (a0 - LD(A, nb[2])) * rdy) + fn * (-r * (LD(A, nb[3]) - a0) * rdy));
      }
      if (k >= 1) {  // bottom face k
        const float fb = g0 * rdz * ri - LD(G, id - plane) * rdz * c.rho_inv[k - 1];
        const float k8 = 0.5f * (kh(id - plane) + khc);
        ab += -c.rho_wext[k] * k8 * rdz * fb;
        khb += 0.5f * fb * (-c.rho_wext[k] * (a0 - LD(A, id - plane)) * rdz);
      }
      if (k + 1 <= nz - 1) {  // top face k+1
        const float ft = LD(G, id + plane) * rdz * c.rho_inv[k + 1] - g0 * rdz * ri;
        const float k8 = 0.5f * (khc + kh(id + plane));
        ab += c.rho_wext[k + 1] * k8 * rdz * ft;
        khb += 0.5f * ft * (-c.rho_wext[k + 1] * (LD(A, id + plane) - a0) * rdz);
      }
      (fld == 0 ? a.x0b.T : a.x0b.q)[id] += ab;
    }
    a.khb[id] = khb;
  }
}

// adjoint of compute_k and of the S^2 / N^2 combination: sbar_ij and N^2 bar at every cell
__global__ void __launch_bounds__(AB) k_smag_s_vjp(Dims d, Cols c, SmagLin l, SmagVjpArgs a) {
  const long long t = (long long)blockIdx.x * AB + threadIdx.x;
  if (t >= d.cells()) return;
  const int id = (int)t, k = (int)(t / d.plane());
  const float ri = c.rho_inv[k], km = LD(l.km, id);
  float s[6], tb[6];
  float kmb = LD(a.khb, id) * kInvPrandtl;
  for (int q = 0; q < 6; ++q) {
    s[q] = LD(l.s[q], id);
    tb[q] = LD(a.tb[q], id);
    kmb += -2.f * s[q] * tb[q];
  }
  if (a.kmkb) a.kmkb[id] = kmb * km;
  const float S2b = kmb * LD(l.kS, id);
  for (int q = 0; q < 6; ++q) a.sb[q][id] = -2.f * km * tb[q] + S2b * (q < 3 ? 4.f : 8.f) * s[q] * (ri * ri);
  a.n2b[id] = -S2b * kInvPrandtl;
}

// adjoint of compute_deformation and compute_nm: winds and theta / qv
__global__ void __launch_bounds__(AB) k_smag_state_vjp(Dims d, Phys ph, Cols c, State s, SmagVjpArgs a) {
  const long long t = (long long)blockIdx.x * AB + threadIdx.x;
  if (t >= d.faces()) return;
  const int nx = d.nx, ny = d.ny, nz = d.nz, plane = d.plane();
  const int i = (int)(t % nx), j = (int)((t / nx) % ny), k = (int)(t / plane);
  const int id = (int)t;
  const float rdx = ph.rdx, rdy = ph.rdy, rdz = ph.rdz;
  auto at = [&](int ii, int jj, int kk) { return (kk * ny + wrapx(jj, ny)) * nx + wrapx(ii, nx); };
  // adjoint of e12 at (u point q, v face jf), level kk
  auto e12b = [&](int q, int jf, int kk) {
    const float* S = a.sb[3];
    return 0.25f * c.rho[kk] * (LD(S, at(q, jf, kk)) + LD(S, at(q - 1, jf - 1, kk)) + LD(S, at(q, jf - 1, kk)) +
                                LD(S, at(q - 1, jf, kk)));
  };
  // adjoint of e13 at (u point q, row jj, w face f) / e23 at (column ii, v face jf, w face f)
  auto e13b = [&](int q, int jj, int f) {
    if (f < 1 || f > nz - 1) return 0.f;
    int ks[4];
    const int n = face_cells(f, nz, ks);
    float acc = 0.f;
    for (int m = 0; m < n; ++m) {
      const int kk = ks[m];
      if (kk < 0 || kk > nz - 1) continue;
      const float w = w_edge(kk, f, nz);
      if (w != 0.f) acc += w * c.rho[kk] * (LD(a.sb[4], at(q - 1, jj, kk)) + LD(a.sb[4], at(q, jj, kk)));
    }
    return acc;
  };
  auto e23b = [&](int ii, int jf, int f) {
    if (f < 1 || f > nz - 1) return 0.f;
    int ks[4];
    const int n = face_cells(f, nz, ks);
    float acc = 0.f;
    for (int m = 0; m < n; ++m) {
      const int kk = ks[m];
      if (kk < 0 || kk > nz - 1) continue;
      const float w = w_edge(kk, f, nz);
      if (w != 0.f) acc += w * c.rho[kk] * (LD(a.sb[5], at(ii, jf - 1, kk)) + LD(a.sb[5], at(ii, jf, kk)));
    }
    return acc;
  };
  // ---- w on face k
  {
    float wb = 0.f;
    if (k >= 1) wb += c.rho[k - 1] * rdz * LD(a.sb[2], id - plane);
    if (k <= nz - 1) wb -= c.rho[k] * rdz * LD(a.sb[2], id);
    wb += 0.5f * rdx * (e13b(i, j, k) - e13b(i + 1, j, k));
    wb += 0.5f * rdy * (e23b(i, j, k) - e23b(i, j + 1, k));
    a.x0b.w[id] += wb;
  }
  if (k >= nz) return;
  const float r = c.rho[k];
  // ---- u (west face of cell i)
  {
    float ub = r * rdx * (LD(a.sb[0], at(i - 1, j, k)) - LD(a.sb[0], id));
    ub += 0.5f * rdy * (e12b(i, j, k) - e12b(i, j + 1, k));
    ub += 0.5f * rdz * (e13b(i, j, k) - e13b(i, j, k + 1));
    a.x0b.u[id] += ub;
  }
  // ---- v (south face of cell j)
  {
    float vb = r * rdy * (LD(a.sb[1], at(i, j - 1, k)) - LD(a.sb[1], id));
    vb += 0.5f * rdx * (e12b(i, j, k) - e12b(i + 1, j, k));
    vb += 0.5f * rdz * (e23b(i, j, k) - e23b(i, j, k + 1));
    a.x0b.v[id] += vb;
  }
  // ---- theta, qv through N^2 = g/dz log(theta_rho_m(f) / theta_rho_m(f-1)) on faces k, k+1
  {
    auto n2fb = [&](int f) {
      if (f < 1 || f > nz - 1) return 0.f;
      int ks[4];
      const int n = face_cells(f, nz, ks);
      float acc = 0.f;
      for (int m = 0; m < n; ++m) {
        const int kk = ks[m];
        if (kk < 0 || kk > nz - 1) continue;
        const float w = w_n2(kk, f, nz);
        if (w != 0.f) acc += w * LD(a.n2b, at(i, j, kk));
      }
      return acc;
    };
    const float T = LD(s.T, id), q = LD(s.q, id);
    const float r1 = (float)kRepsm1;
    const float trm = (ph.theta_ref + T) * (1.f + r1 * q);
    const float trmb = (float)kG * rdz * (n2fb(k) - n2fb(k + 1)) / trm;
    a.x0b.T[id] += trmb * (1.f + r1 * q);
    a.x0b.q[id] += trmb * (ph.theta_ref + T) * r1;
  }
}

}  // namespace

cudaError_t launch_acoustic_vjp(const Dims& d, const Phys& ph, const Cols& c, const AcousticVjpArgs& a, float dtau,
                                cudaStream_t st, const cudaAccessPolicyWindow* win) {
  constexpr int V = ACOUSTIC_VJP_VEC;
  if (d.nx % V == 0) {
    // small blocks: many registers per thread (a register cap that made the 4-wide kernel spill
    // float4 values faulted with a misaligned address)
    dim3 b(16, 4, 1);
    dim3 g((d.nx / V + 15) / 16, (d.ny + 3) / 4, d.nz);
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
      return cudaLaunchKernelEx(&cfg, k_acoustic_vjpv<V>, d, ph, c, a, dtau);
    }
    k_acoustic_vjpv<V><<<g, b, 0, st>>>(d, ph, c, a, dtau);
    return cudaGetLastError();
  }
  const unsigned g = (unsigned)((d.cells() + AB - 1) / AB);
  k_acoustic_vjp<<<g, AB, 0, st>>>(d, ph, c, a, dtau);
  return cudaGetLastError();
}

cudaError_t launch_stage_pointwise_vjp(const Dims& d, const Phys& ph, const Cols& c, const StageVjpArgs& a,
                                       cudaStream_t st) {
  const unsigned g = (unsigned)((d.faces() + AB - 1) / AB);
  k_stage_pointwise_vjp<<<g, AB, 0, st>>>(d, ph, c, a);
  return cudaGetLastError();
}

cudaError_t launch_massdiv_vjp(const Dims& d, const Phys& ph, const Cols& c, const float* divb, State xsb,
                               cudaStream_t st, State x0b) {
  const unsigned g = (unsigned)((d.faces() + AB - 1) / AB);
  k_massdiv_vjp<<<g, AB, 0, st>>>(d, ph, c, divb, xsb, x0b);
  return cudaGetLastError();
}

// out += scale * sum(x): per-thread FP64 partial sums, a block reduction, one atomic a block
__global__ void __launch_bounds__(256) k_sum_scaled(long long n, const float* __restrict__ x, double scale,
                                                    double* __restrict__ out) {
  __shared__ double part[8];
  double acc = 0.0;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    acc += (double)x[i];
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int wv = 0; wv < 8; ++wv) s += part[wv];
    atomicAdd(out, scale * s);
  }
}

cudaError_t launch_sum_scaled(long long n, const float* x, double scale, double* out, cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  long long b = (n + 255) / 256;
  if (b > 1024) b = 1024;
  k_sum_scaled<<<(unsigned)b, 256, 0, st>>>(n, x, scale, out);
  return cudaGetLastError();
}

cudaError_t launch_smag_vjp(const Dims& d, const Phys& ph, const Cols& c, State x0, const SmagLin& l,
                            const SmagVjpArgs& a, cudaStream_t st) {
  const unsigned gc = (unsigned)((d.cells() + AB - 1) / AB), gf = (unsigned)((d.faces() + AB - 1) / AB);
  k_smag_lin<<<gc, AB, 0, st>>>(d, ph, c, x0, l);
  k_smag_tau_vjp<<<gc, AB, 0, st>>>(d, ph, c, x0, l, a);
  k_smag_s_vjp<<<gc, AB, 0, st>>>(d, c, l, a);
  k_smag_state_vjp<<<gf, AB, 0, st>>>(d, ph, c, x0, a);
  return cudaGetLastError();
}

cudaError_t launch_adv_vjp(const Dims& d, const Phys& ph, const Cols& c, const AdvVjpArgs& a, cudaStream_t st) {
  const unsigned g = (unsigned)((d.faces() + AB - 1) / AB);
  k_adv_face_vjp<0><<<g, AB, 0, st>>>(d, ph, c, a);
  k_adv_gather_vjp<0><<<g, AB, 0, st>>>(d, ph, c, a);
  k_adv_face_vjp<1><<<g, AB, 0, st>>>(d, ph, c, a);
  k_adv_gather_vjp<1><<<g, AB, 0, st>>>(d, ph, c, a);
  k_adv_face_vjp<2><<<g, AB, 0, st>>>(d, ph, c, a);
  k_adv_gather_vjp<2><<<g, AB, 0, st>>>(d, ph, c, a);
  return cudaGetLastError();
}

}  // namespace lexgb

namespace lexgb {
namespace {
__global__ void k_axpy(float* __restrict__ y, const float* __restrict__ x, size_t n) {
  for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x)
    y[t] += x[t];
}
}  // namespace

cudaError_t launch_axpy(float* y, const float* x, size_t n, cudaStream_t st) {
  const unsigned g = (unsigned)((n + 255) / 256 < 8192 ? (n + 255) / 256 : 8192);
  k_axpy<<<g > 0 ? g : 1, 256, 0, st>>>(y, x, n);
  return cudaGetLastError();
}
}  // namespace lexgb

namespace lexgb {
namespace {
__global__ void k_shift(float* __restrict__ y, float c, size_t n) {
  for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x)
    y[t] += c;
}
}  // namespace

cudaError_t launch_shift(float* y, float c, size_t n, cudaStream_t st) {
  const unsigned g = (unsigned)((n + 255) / 256 < 8192 ? (n + 255) / 256 : 8192);
  k_shift<<<g > 0 ? g : 1, 256, 0, st>>>(y, c, n);
  return cudaGetLastError();
}
}  // namespace lexgb
