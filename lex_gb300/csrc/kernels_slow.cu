// kernels_slow.cu - per-stage diagnostics feeding the WENO kernels and the acoustic loop:
//   k_div_trho  mass divergence div(rho0 u) (get_divergence, advection.py:200-226) and the
//               density potential temperature theta (1 + reps qv) / (1 + qv)
//               (one_step_integration.py:269).  One thread per cell.
// The WENO advection itself lives in kernels_weno.cu.
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

}  // namespace

cudaError_t launch_div_trho(const Dims& d, const Phys& ph, const Cols& c, State in, float* div, float* trho,
                            cudaStream_t st) {
  k_div_trho<<<grid_for(d, d.nz), dim3(BX, BY, BZ), 0, st>>>(d, ph, c, in, div, trho);
  return cudaGetLastError();
}

}  // namespace lexgb
