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
  dim3 g((d.nx + BX - 1) / BX, (d.ny + BY - 1) / BY, (d.nz + BZ - 1) / BZ);
  k_acoustic<<<g, dim3(BX, BY, BZ), 0, st>>>(d, ph, c, in, out, dtau);
  return cudaGetLastError();
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
