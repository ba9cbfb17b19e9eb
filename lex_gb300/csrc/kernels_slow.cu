// kernels_slow.cu - slow-mode (advective) tendencies of one RK stage.
//
//   k_div_trho     mass divergence div(rho0 u) (get_divergence, advection.py:200-226) and the
//                  density potential temperature used by the acoustic loop
//                  (one_step_integration.py:269)
//   k_adv_scalars  WENO5-Z flux-form advection of theta and qv (advection_scalar,
//                  advection.py:9-34; fluxes :305-516) fused with the Euler stage update
//                  theta_next = theta^0 + dt_s (adv + sgs) (one_step_integration.py:285-296, :450-466)
//   k_adv_u/_v/_w  momentum advection (advection.py:37-149; fluxes :561-1281) fused with the
//                  slow right-hand sides rhs_u/v/w = adv + Coriolis + buoyancy + SGS
//                  (one_step_integration.py:258-263)
// One thread per output point; stencil neighbours come through the read-only path.
#include "lexgb_internal.cuh"

namespace lexgb {

namespace {

constexpr int BX = 32, BY = 4, BZ = 2;

inline dim3 grid_for(const Dims& d, int nzz) {
  return dim3((d.nx + BX - 1) / BX, (d.ny + BY - 1) / BY, (nzz + BZ - 1) / BZ);
}

#define LD(p, idx) __ldg((p) + (idx))

__global__ void __launch_bounds__(BX* BY* BZ) k_div_trho(Dims d, Phys ph, Cols c, State s, float* __restrict__ div,
                                                       float* __restrict__ trho) {
  const int i = blockIdx.x * BX + threadIdx.x, j = blockIdx.y * BY + threadIdx.y, k = blockIdx.z * BZ + threadIdx.z;
  if (i >= d.nx || j >= d.ny || k >= d.nz) return;
  const int ip = wrap(i + 1, d.nx), jp = wrap(j + 1, d.ny);
  const int id = d.at(i, j, k);
  const float r = c.rho[k];
  const float dvx = (r * LD(s.u, d.at(ip, j, k)) - r * LD(s.u, id)) * ph.rdx;
  const float dvy = (r * LD(s.v, d.at(i, jp, k)) - r * LD(s.v, id)) * ph.rdy;
  const float dvz = (c.rho_face0[k + 1] * LD(s.w, d.at(i, j, k + 1)) - c.rho_face0[k] * LD(s.w, id)) * ph.rdz;
  div[id] = dvx + dvy + dvz;
  trho[id] = theta_rho(LD(s.T, id), LD(s.q, id), ph.theta_ref);
}

// Flux-form advection of one scalar at cell (i, j, k); returns the advective tendency.
__device__ __forceinline__ float scalar_tendency(const Dims& d, const Phys& ph, const Cols& c, const State& s,
                                                 const float* __restrict__ f, const float* __restrict__ div, int i,
                                                 int j, int k, float eps) {
  const int nx = d.nx, ny = d.ny, nz = d.nz;
  const float r = c.rho[k];
  float x[7], y[7];
#pragma unroll
  for (int o = 0; o < 7; ++o) {
    x[o] = LD(f, d.at(wrap(i - 3 + o, nx), j, k));
    y[o] = LD(f, d.at(i, wrap(j - 3 + o, ny), k));
  }
  // x faces i (west) and i+1 (east)
  const float mw = r * LD(s.u, d.at(i, j, k));
  const float me = r * LD(s.u, d.at(wrap(i + 1, nx), j, k));
  const float fw = weno_flux(mw, x[0], x[1], x[2], x[3], x[4], x[5], eps);
  const float fe = weno_flux(me, x[1], x[2], x[3], x[4], x[5], x[6], eps);
  const float ms = r * LD(s.v, d.at(i, j, k));
  const float mn = r * LD(s.v, d.at(i, wrap(j + 1, ny), k));
  const float fs = weno_flux(ms, y[0], y[1], y[2], y[3], y[4], y[5], eps);
  const float fn = weno_flux(mn, y[1], y[2], y[3], y[4], y[5], y[6], eps);
  auto colv = [&](int kk) { return LD(f, d.at(i, j, kk)); };
  float fz[2];
#pragma unroll
  for (int o = 0; o < 2; ++o) {
    const int fk = k + o;
    const float m = c.rho_face[fk] * LD(s.w, d.at(i, j, fk));
    fz[o] = (fk == 0) ? 0.f : vflux(m, colv, fk, nz, eps);
  }
  const float conv = -((fe - fw) * ph.rdx + (fn - fs) * ph.rdy + (fz[1] - fz[0]) * ph.rdz);
  const int id = d.at(i, j, k);
  return (conv + x[3] * LD(div, id)) / r;
}

__global__ void __launch_bounds__(BX* BY* BZ) k_adv_scalars(Dims d, Phys ph, Cols c, State s,
                                                          const float* __restrict__ div, const float* T0,
                                                          const float* q0, Sgs sgs, float dts,
                                                          SlowOut out) {
  const int i = blockIdx.x * BX + threadIdx.x, j = blockIdx.y * BY + threadIdx.y, k = blockIdx.z * BZ + threadIdx.z;
  if (i >= d.nx || j >= d.ny || k >= d.nz) return;
  const int id = d.at(i, j, k);
  const float aT = scalar_tendency(d, ph, c, s, s.T, div, i, j, k, kWepsTheta);
  const float aq = scalar_tendency(d, ph, c, s, s.q, div, i, j, k, kWepsQv);
  // T0/q0 may alias the outputs (the last stage updates the step's initial state in place):
  // each element is read and then written by the same thread only, so plain loads are used.
  float Tn = T0[id] + aT * dts;
  float qn = q0[id] + aq * dts;
  float dT = aT, dq = aq;
  if (sgs.T) {
    const float st = LD(sgs.T, id), sq = LD(sgs.q, id);
    Tn = Tn + st * dts;
    qn = qn + sq * dts;
    dT = dT + st;
    dq = dq + sq;
  }
  if (out.T_next) out.T_next[id] = Tn;
  if (out.q_next) out.q_next[id] = qn;
  if (out.dT) out.dT[id] = dT;
  if (out.dq) out.dq[id] = dq;
}

__global__ void __launch_bounds__(BX* BY* BZ) k_adv_u(Dims d, Phys ph, Cols c, State s, const float* __restrict__ div,
                                                    const float* __restrict__ sgs_u, float* __restrict__ Ru) {
  const int i = blockIdx.x * BX + threadIdx.x, j = blockIdx.y * BY + threadIdx.y, k = blockIdx.z * BZ + threadIdx.z;
  if (i >= d.nx || j >= d.ny || k >= d.nz) return;
  const int nx = d.nx, ny = d.ny, nz = d.nz;
  const float eps = kWepsMom;
  const float r = c.rho[k];
  const int im = wrap(i - 1, nx);
  float x[7], y[7];
#pragma unroll
  for (int o = 0; o < 7; ++o) {
    x[o] = LD(s.u, d.at(wrap(i - 3 + o, nx), j, k));
    y[o] = LD(s.u, d.at(i, wrap(j - 3 + o, ny), k));
  }
  // x flux at the cells west (i-1) and east (i) of u(i)
  const float fw = weno_flux(0.5f * (x[2] + x[3]) * r, x[0], x[1], x[2], x[3], x[4], x[5], eps);
  const float fe = weno_flux(0.5f * (x[3] + x[4]) * r, x[1], x[2], x[3], x[4], x[5], x[6], eps);
  // y flux at the corners south (face j) and north (face j+1) of u(i, j)
  const int jp = wrap(j + 1, ny);
  const float ms = 0.5f * (r * LD(s.v, d.at(im, j, k)) + r * LD(s.v, d.at(i, j, k)));
  const float mn = 0.5f * (r * LD(s.v, d.at(im, jp, k)) + r * LD(s.v, d.at(i, jp, k)));
  const float fs = weno_flux(ms, y[0], y[1], y[2], y[3], y[4], y[5], eps);
  const float fn = weno_flux(mn, y[1], y[2], y[3], y[4], y[5], y[6], eps);
  auto colv = [&](int kk) { return LD(s.u, d.at(i, j, kk)); };
  float fz[2];
#pragma unroll
  for (int o = 0; o < 2; ++o) {
    const int fk = k + o;
    const float rf = c.rho_face[fk];
    const float m = 0.5f * (rf * LD(s.w, d.at(im, j, fk)) + rf * LD(s.w, d.at(i, j, fk)));
    fz[o] = (fk == 0) ? 0.f : vflux(m, colv, fk, nz, eps);
  }
  const float conv = -((fe - fw) * ph.rdx + (fn - fs) * ph.rdy + (fz[1] - fz[0]) * ph.rdz);
  const float d8u = 0.5f * (LD(div, d.at(im, j, k)) + LD(div, d.at(i, j, k)));
  float R = (conv + x[3] * d8u) / r;
  if (ph.cor_opt) {  // + fv (pressure_gradient_coriolis.py:80-95)
    const float fv = ph.f_cor * 0.25f * (LD(s.v, d.at(im, j, k)) + LD(s.v, d.at(im, jp, k)) +
                                         LD(s.v, d.at(i, j, k)) + LD(s.v, d.at(i, jp, k)));
    R = R + fv;
  }
  if (sgs_u) R = R + LD(sgs_u, d.at(i, j, k));
  Ru[d.at(i, j, k)] = R;
}

__global__ void __launch_bounds__(BX* BY* BZ) k_adv_v(Dims d, Phys ph, Cols c, State s, const float* __restrict__ div,
                                                    const float* __restrict__ sgs_v, float* __restrict__ Rv) {
  const int i = blockIdx.x * BX + threadIdx.x, j = blockIdx.y * BY + threadIdx.y, k = blockIdx.z * BZ + threadIdx.z;
  if (i >= d.nx || j >= d.ny || k >= d.nz) return;
  const int nx = d.nx, ny = d.ny, nz = d.nz;
  const float eps = kWepsMom;
  const float r = c.rho[k];
  const int jm = wrap(j - 1, ny);
  float x[7], y[7];
#pragma unroll
  for (int o = 0; o < 7; ++o) {
    x[o] = LD(s.v, d.at(wrap(i - 3 + o, nx), j, k));
    y[o] = LD(s.v, d.at(i, wrap(j - 3 + o, ny), k));
  }
  // x flux at the corners west (face i) and east (face i+1) of v(i, j)
  const int ip = wrap(i + 1, nx);
  const float mw = 0.5f * (r * LD(s.u, d.at(i, jm, k)) + r * LD(s.u, d.at(i, j, k)));
  const float me = 0.5f * (r * LD(s.u, d.at(ip, jm, k)) + r * LD(s.u, d.at(ip, j, k)));
  const float fw = weno_flux(mw, x[0], x[1], x[2], x[3], x[4], x[5], eps);
  const float fe = weno_flux(me, x[1], x[2], x[3], x[4], x[5], x[6], eps);
  // y flux at the cells south (j-1) and north (j) of v(j)
  const float fs = weno_flux(0.5f * (y[2] + y[3]) * r, y[0], y[1], y[2], y[3], y[4], y[5], eps);
  const float fn = weno_flux(0.5f * (y[3] + y[4]) * r, y[1], y[2], y[3], y[4], y[5], y[6], eps);
  auto colv = [&](int kk) { return LD(s.v, d.at(i, j, kk)); };
  float fz[2];
#pragma unroll
  for (int o = 0; o < 2; ++o) {
    const int fk = k + o;
    const float rf = c.rho_face[fk];
    const float m = 0.5f * (rf * LD(s.w, d.at(i, jm, fk)) + rf * LD(s.w, d.at(i, j, fk)));
    fz[o] = (fk == 0) ? 0.f : vflux(m, colv, fk, nz, eps);
  }
  const float conv = -((fe - fw) * ph.rdx + (fn - fs) * ph.rdy + (fz[1] - fz[0]) * ph.rdz);
  const float d8v = 0.5f * (LD(div, d.at(i, jm, k)) + LD(div, d.at(i, j, k)));
  float R = (conv + y[3] * d8v) / r;
  if (ph.cor_opt) {  // - fu (pressure_gradient_coriolis.py:80-113)
    float fu = 0.25f * (LD(s.u, d.at(i, jm, k)) + LD(s.u, d.at(i, j, k)) + LD(s.u, d.at(ip, jm, k)) +
                        LD(s.u, d.at(ip, j, k)));
    fu = ph.cor_opt == 2 ? ph.f_cor * (fu - 1.0f) : ph.f_cor * fu;
    R = R - fu;
  }
  if (sgs_v) R = R + LD(sgs_v, d.at(i, j, k));
  Rv[d.at(i, j, k)] = R;
}

__global__ void __launch_bounds__(BX* BY* BZ) k_adv_w(Dims d, Phys ph, Cols c, State s, const float* __restrict__ div,
                                                    const float* __restrict__ sgs_w, float* __restrict__ Rw, int mode) {
  const int i = blockIdx.x * BX + threadIdx.x, j = blockIdx.y * BY + threadIdx.y, f = blockIdx.z * BZ + threadIdx.z;
  const int nx = d.nx, ny = d.ny, nz = d.nz;
  if (i >= nx || j >= ny || f > nz) return;
  const float eps = kWepsMom;
  const int id = d.at(i, j, f);
  float adv = 0.f;
  if (mode != 2 && f > 0 && f < nz) {
    float x[7], y[7];
#pragma unroll
    for (int o = 0; o < 7; ++o) {
      x[o] = LD(s.w, d.at(wrap(i - 3 + o, nx), j, f));
      y[o] = LD(s.w, d.at(i, wrap(j - 3 + o, ny), f));
    }
    const float rl = c.rho[f - 1], ru = c.rho[f];
    const int ip = wrap(i + 1, nx), jp = wrap(j + 1, ny);
    // x flux at u points i and i+1 on face f
    const float mw = 0.5f * (rl * LD(s.u, d.at(i, j, f - 1)) + ru * LD(s.u, d.at(i, j, f)));
    const float me = 0.5f * (rl * LD(s.u, d.at(ip, j, f - 1)) + ru * LD(s.u, d.at(ip, j, f)));
    const float fw = weno_flux(mw, x[0], x[1], x[2], x[3], x[4], x[5], eps);
    const float fe = weno_flux(me, x[1], x[2], x[3], x[4], x[5], x[6], eps);
    const float ms = 0.5f * (rl * LD(s.v, d.at(i, j, f - 1)) + ru * LD(s.v, d.at(i, j, f)));
    const float mn = 0.5f * (rl * LD(s.v, d.at(i, jp, f - 1)) + ru * LD(s.v, d.at(i, jp, f)));
    const float fs = weno_flux(ms, y[0], y[1], y[2], y[3], y[4], y[5], eps);
    const float fn = weno_flux(mn, y[1], y[2], y[3], y[4], y[5], y[6], eps);
    // z flux at the cells below (f-1) and above (f) the face, w column has nz+1 entries
    auto colw = [&](int kk) { return LD(s.w, d.at(i, j, kk)); };
    float fz[2];
#pragma unroll
    for (int o = 0; o < 2; ++o) {
      const int cc = f - 1 + o;
      const float m = 0.5f * (colw(cc) + colw(cc + 1)) * c.rho[cc];
      fz[o] = vflux(m, colw, cc + 1, nz + 1, eps);
    }
    const float conv = -((fe - fw) * ph.rdx + (fn - fs) * ph.rdy + (fz[1] - fz[0]) * ph.rdz);
    const float d8w = 0.5f * (LD(div, d.at(i, j, f - 1)) + LD(div, d.at(i, j, f)));
    const float r8w = 0.5f * (rl + ru);
    adv = (conv + x[3] * d8w) / r8w;
  }
  if (mode == 1) {
    Rw[id] = adv;
    return;
  }
  // buoyancy at the face (interpolate_scalar2w with end extrapolation, pressure_equations.py:123-159)
  auto b = [&](int kk) { return buoyancy_at(LD(s.T, d.at(i, j, kk)), LD(s.q, d.at(i, j, kk)), kk, c); };
  float b8w;
  if (f == 0)
    b8w = 1.875f * b(0) - 1.25f * b(1) + 0.375f * b(2);
  else if (f == nz)
    b8w = 1.875f * b(nz - 1) - 1.25f * b(nz - 2) + 0.375f * b(nz - 3);
  else
    b8w = 0.5f * (b(f - 1) + b(f));
  if (mode == 2) {
    Rw[id] = b8w;
    return;
  }
  float R = adv + b8w;
  if (sgs_w) R = R + LD(sgs_w, id);
  Rw[id] = R;
}

}  // namespace

cudaError_t launch_div_trho(const Dims& d, const Phys& ph, const Cols& c, State in, float* div, float* trho,
                            cudaStream_t st) {
  k_div_trho<<<grid_for(d, d.nz), dim3(BX, BY, BZ), 0, st>>>(d, ph, c, in, div, trho);
  return cudaGetLastError();
}

cudaError_t launch_adv_scalars(const Dims& d, const Phys& ph, const Cols& c, State in, const float* div,
                               const float* T0, const float* q0, Sgs sgs, float dts, SlowOut out, cudaStream_t st) {
  k_adv_scalars<<<grid_for(d, d.nz), dim3(BX, BY, BZ), 0, st>>>(d, ph, c, in, div, T0, q0, sgs, dts, out);
  return cudaGetLastError();
}

cudaError_t launch_adv_u(const Dims& d, const Phys& ph, const Cols& c, State in, const float* div,
                         const float* sgs_u, float* Ru, cudaStream_t st) {
  k_adv_u<<<grid_for(d, d.nz), dim3(BX, BY, BZ), 0, st>>>(d, ph, c, in, div, sgs_u, Ru);
  return cudaGetLastError();
}

cudaError_t launch_adv_v(const Dims& d, const Phys& ph, const Cols& c, State in, const float* div,
                         const float* sgs_v, float* Rv, cudaStream_t st) {
  k_adv_v<<<grid_for(d, d.nz), dim3(BX, BY, BZ), 0, st>>>(d, ph, c, in, div, sgs_v, Rv);
  return cudaGetLastError();
}

cudaError_t launch_adv_w(const Dims& d, const Phys& ph, const Cols& c, State in, const float* div,
                         const float* sgs_w, float* Rw, int mode, cudaStream_t st) {
  k_adv_w<<<grid_for(d, d.nz + 1), dim3(BX, BY, BZ), 0, st>>>(d, ph, c, in, div, sgs_w, Rw, mode);
  return cudaGetLastError();
}

}  // namespace lexgb
