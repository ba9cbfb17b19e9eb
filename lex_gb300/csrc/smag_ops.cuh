// smag_ops.cuh - strain-rate edges, N^2 faces and the end extrapolation of the Smagorinsky
// closure (turbulence.py:298-427), shared by the forward kernels and their reverse mode.
#pragma once
#include "lexgb_internal.cuh"

namespace lexgb {
namespace smag {

#define SMAG_LD(p, idx) __ldg((p) + (idx))

__device__ __forceinline__ float ext3(float a, float b, float c) { return 1.875f * a - 1.25f * b + 0.375f * c; }

// strain-rate edges: e12 at (u point q, v face jf); e13 at (u point q, w face f); e23 at (v face jf, w face f)
__device__ __forceinline__ float e12(const Dims& d, const Phys& ph, const State& s, int q, int jf, int k) {
  const int qw = wrap(q, d.nx), jj = wrap(jf, d.ny);
  const float dudy = (SMAG_LD(s.u, d.at(qw, jj, k)) - SMAG_LD(s.u, d.at(qw, wrap(jf - 1, d.ny), k))) * ph.rdy;
  const float dvdx = (SMAG_LD(s.v, d.at(qw, jj, k)) - SMAG_LD(s.v, d.at(wrap(q - 1, d.nx), jj, k))) * ph.rdx;
  return 0.5f * (dudy + dvdx);
}

__device__ __forceinline__ float e13(const Dims& d, const Phys& ph, const State& s, int q, int j, int f) {
  const int qw = wrap(q, d.nx);
  const float dudz = (SMAG_LD(s.u, d.at(qw, j, f)) - SMAG_LD(s.u, d.at(qw, j, f - 1))) * ph.rdz;
  const float dwdx = (SMAG_LD(s.w, d.at(qw, j, f)) - SMAG_LD(s.w, d.at(wrap(q - 1, d.nx), j, f))) * ph.rdx;
  return 0.5f * (dudz + dwdx);
}

__device__ __forceinline__ float e23(const Dims& d, const Phys& ph, const State& s, int i, int jf, int f) {
  const int jj = wrap(jf, d.ny);
  const float dvdz = (SMAG_LD(s.v, d.at(i, jj, f)) - SMAG_LD(s.v, d.at(i, jj, f - 1))) * ph.rdz;
  const float dwdy = (SMAG_LD(s.w, d.at(i, jj, f)) - SMAG_LD(s.w, d.at(i, wrap(jf - 1, d.ny), f))) * ph.rdy;
  return 0.5f * (dvdz + dwdy);
}

// log(theta_rho_m(f) / theta_rho_m(f-1)) * g / dz on interior face f, theta_rho_m = theta (1 + repsm1 qv),
// written as log1p(difference / lower) with the difference formed from T = theta - theta_ref.
__device__ __forceinline__ float n2_face(const Dims& d, const Phys& ph, const State& s, int i, int j, int f) {
  const int a = d.at(i, j, f), b = d.at(i, j, f - 1);
  const float Ta = SMAG_LD(s.T, a), Tb = SMAG_LD(s.T, b), qa = SMAG_LD(s.q, a), qb = SMAG_LD(s.q, b);
  const float r1 = (float)kRepsm1;
  const float lower = (ph.theta_ref + Tb) * (1.f + r1 * qb);
  const float diff = (Ta - Tb) * (1.f + r1 * qa) + (ph.theta_ref + Tb) * r1 * (qa - qb);
  return log1pf(diff / lower) * ph.rdz * (float)kG;
}


#undef SMAG_LD

}  // namespace smag
}  // namespace lexgb
