// kernels_smag.cu - Smagorinsky SGS tendencies, once per RK3 big step from the step's
// initial state (one_step_integration.py:57-76).
//
//   k_smag_a  rho-weighted strain rates S_ij at cell centres (compute_deformation,
//             turbulence.py:298-388), N^2 (compute_nm, :391-427), K_m and K_h (compute_k,
//             :430-446); writes tau_ij = -2 K_m S_ij and K_h.
//   k_smag_b  stress divergence on u, v, w points and the flux-form scalar diffusion of
//             theta and qv (compute_smag, turbulence.py:9-111, with compute_scalar_gradient
//             :474-494 and stagger_scalar :497-504).
#include "smag_ops.cuh"

namespace lexgb {

namespace {

constexpr int BX = 32, BY = 4, BZ = 2;
#define LD(p, idx) __ldg((p) + (idx))
using namespace smag;

__global__ void __launch_bounds__(BX* BY* BZ) k_smag_a(Dims d, Phys ph, Cols c, State s, SmagTau o) {
  const int i = blockIdx.x * BX + threadIdx.x, j = blockIdx.y * BY + threadIdx.y, k = blockIdx.z * BZ + threadIdx.z;
  const int nx = d.nx, ny = d.ny, nz = d.nz;
  if (i >= nx || j >= ny || k >= nz) return;
  const int id = d.at(i, j, k);
  const float r = c.rho[k];
  const int ip = wrap(i + 1, nx), jp = wrap(j + 1, ny);
  const float s11 = r * (LD(s.u, d.at(ip, j, k)) - LD(s.u, id)) * ph.rdx;
  const float s22 = r * (LD(s.v, d.at(i, jp, k)) - LD(s.v, id)) * ph.rdy;
  const float s33 = r * (LD(s.w, d.at(i, j, k + 1)) - LD(s.w, id)) * ph.rdz;
  const float s12 =
      r * (0.25f * (e12(d, ph, s, i, j, k) + e12(d, ph, s, i + 1, j + 1, k) + e12(d, ph, s, i, j + 1, k) +
                    e12(d, ph, s, i + 1, j, k)));
  float s13, s23;
  if (k == 0) {
    const float bw = ext3(e13(d, ph, s, i, j, 1), e13(d, ph, s, i, j, 2), e13(d, ph, s, i, j, 3));
    const float be = ext3(e13(d, ph, s, i + 1, j, 1), e13(d, ph, s, i + 1, j, 2), e13(d, ph, s, i + 1, j, 3));
    s13 = 0.5f * (be + bw);
    const float bs = ext3(e23(d, ph, s, i, j, 1), e23(d, ph, s, i, j, 2), e23(d, ph, s, i, j, 3));
    const float bn = ext3(e23(d, ph, s, i, j + 1, 1), e23(d, ph, s, i, j + 1, 2), e23(d, ph, s, i, j + 1, 3));
    s23 = 0.5f * (bn + bs);
  } else if (k == nz - 1) {
    const int f1 = nz - 1, f2 = nz - 2, f3 = nz - 3;
    const float tw = ext3(e13(d, ph, s, i, j, f1), e13(d, ph, s, i, j, f2), e13(d, ph, s, i, j, f3));
    const float te = ext3(e13(d, ph, s, i + 1, j, f1), e13(d, ph, s, i + 1, j, f2), e13(d, ph, s, i + 1, j, f3));
    s13 = 0.5f * (te + tw);
    const float ts = ext3(e23(d, ph, s, i, j, f1), e23(d, ph, s, i, j, f2), e23(d, ph, s, i, j, f3));
    const float tn = ext3(e23(d, ph, s, i, j + 1, f1), e23(d, ph, s, i, j + 1, f2), e23(d, ph, s, i, j + 1, f3));
    s23 = 0.5f * (tn + ts);
  } else {
    s13 = 0.25f * (e13(d, ph, s, i, j, k) + e13(d, ph, s, i + 1, j, k + 1) + e13(d, ph, s, i, j, k + 1) +
                   e13(d, ph, s, i + 1, j, k));
    s23 = 0.25f * (e23(d, ph, s, i, j, k) + e23(d, ph, s, i, j + 1, k + 1) + e23(d, ph, s, i, j, k + 1) +
                   e23(d, ph, s, i, j + 1, k));
  }
  s13 = r * s13;
  s23 = r * s23;
  const float ri = c.rho_inv[k];   // products with the correctly rounded reciprocal instead of divisions
  const float s2 = (2.f * (s11 * s11 + s22 * s22 + s33 * s33) + 4.f * (s12 * s12 + s13 * s13 + s23 * s23)) * (ri * ri);
  float n2;
  if (k == 0)
    n2 = ext3(n2_face(d, ph, s, i, j, 1), n2_face(d, ph, s, i, j, 2), n2_face(d, ph, s, i, j, 3));
  else if (k == nz - 1)
    n2 = ext3(n2_face(d, ph, s, i, j, nz - 1), n2_face(d, ph, s, i, j, nz - 2), n2_face(d, ph, s, i, j, nz - 3));
  else
    n2 = 0.5f * (n2_face(d, ph, s, i, j, k) + n2_face(d, ph, s, i, j, k + 1));
  float s2n2 = s2 - n2 * kInvPrandtl;
  s2n2 = s2n2 > 0.f ? s2n2 : 0.f;
  const float km = ph.smag_l2 * sqrtf(s2n2);
  o.t11[id] = -2.f * km * s11;
  o.t22[id] = -2.f * km * s22;
  o.t33[id] = -2.f * km * s33;
  o.t12[id] = -2.f * km * s12;
  o.t13[id] = -2.f * km * s13;
  o.t23[id] = -2.f * km * s23;
  o.kh[id] = km * kInvPrandtl;
  if (o.n2) o.n2[id] = n2;
  if (o.km) o.km[id] = km;
}

// interpolate_scalar2w_0 of a cell field g(level) onto face f: zero at the ends
template <class F>
__device__ __forceinline__ float to_w0(const F& g, int f, int nz) {
  return (f <= 0 || f >= nz) ? 0.f : 0.5f * (g(f - 1) + g(f));
}

__global__ void __launch_bounds__(BX* BY* BZ) k_smag_b(Dims d, Phys ph, Cols c, State s, SmagTau t, SgsOut o) {
  const int i = blockIdx.x * BX + threadIdx.x, j = blockIdx.y * BY + threadIdx.y, k = blockIdx.z * BZ + threadIdx.z;
  const int nx = d.nx, ny = d.ny, nz = d.nz;
  if (i >= nx || j >= ny || k > nz) return;
  const int im = wrap(i - 1, nx), ip = wrap(i + 1, nx), jm = wrap(j - 1, ny), jp = wrap(j + 1, ny);
  const float rdx = ph.rdx, rdy = ph.rdy, rdz = ph.rdz;
  auto T = [&](const float* a, int ii, int jj, int kk) { return LD(a, d.at(ii, jj, kk)); };
  // ---------------------------------------------------------------- w point (face k)
  {
    float sw = 0.f;
    if (k > 0 && k < nz) {
      const float d33 = (T(t.t33, i, j, k) - T(t.t33, i, j, k - 1)) * rdz;
      auto g13 = [&](int kk) { return (T(t.t13, ip, j, kk) - T(t.t13, im, j, kk)) * (0.5f * rdx); };
      auto g23 = [&](int kk) { return (T(t.t23, i, jp, kk) - T(t.t23, i, jm, kk)) * (0.5f * rdy); };
      sw = -(to_w0(g13, k, nz) + to_w0(g23, k, nz) + d33) * c.rho_wext_inv[k];
    }
    o.w[d.at(i, j, k)] = sw;
  }
  if (k >= nz) return;
  const int id = d.at(i, j, k);
  const float r = c.rho[k], ri = c.rho_inv[k];
  // ---------------------------------------------------------------- u point (west face of cell i)
  {
    const float d11 = (T(t.t11, i, j, k) - T(t.t11, im, j, k)) * rdx;
    auto d12v = [&](int cc, int jf) {  // d tau12 / dy on the v face jf of column cc
      const int cw = wrap(cc, nx), jw = wrap(jf, ny);
      return (T(t.t12, cw, jw, k) - T(t.t12, cw, wrap(jf - 1, ny), k)) * rdy;
    };
    const float d12 = 0.25f * (d12v(i - 1, j) + d12v(i, j + 1) + d12v(i - 1, j + 1) + d12v(i, j));
    auto d13s = [&](int cc) {  // d tau13 / dz at cell level k of column cc, tau13 taken to faces with zero ends
      auto g = [&](int kk) { return T(t.t13, cc, j, kk); };
      return (to_w0(g, k + 1, nz) - to_w0(g, k, nz)) * rdz;
    };
    const float d13 = 0.5f * (d13s(im) + d13s(i));
    o.u[id] = -(d11 + d12 + d13) * ri;
  }
  // ---------------------------------------------------------------- v point (south face of cell j)
  {
    const float d22 = (T(t.t22, i, j, k) - T(t.t22, i, jm, k)) * rdy;
    auto d12u = [&](int q, int rr) {  // d tau12 / dx on the u face q of row rr
      const int qw = wrap(q, nx), rw = wrap(rr, ny);
      return (T(t.t12, qw, rw, k) - T(t.t12, wrap(q - 1, nx), rw, k)) * rdx;
    };
    const float d12 = 0.25f * (d12u(i, j - 1) + d12u(i + 1, j) + d12u(i, j) + d12u(i + 1, j - 1));
    auto d23s = [&](int rr) {
      auto g = [&](int kk) { return T(t.t23, i, rr, kk); };
      return (to_w0(g, k + 1, nz) - to_w0(g, k, nz)) * rdz;
    };
    const float d23 = 0.5f * (d23s(jm) + d23s(j));
    o.v[id] = -(d12 + d22 + d23) * ri;
  }
  // ---------------------------------------------------------------- scalars (cell)
  {
    auto kh8u = [&](int q) { return 0.5f * (T(t.kh, wrap(q, nx), j, k) + T(t.kh, wrap(q - 1, nx), j, k)); };
    auto kh8v = [&](int rr) { return 0.5f * (T(t.kh, i, wrap(rr, ny), k) + T(t.kh, i, wrap(rr - 1, ny), k)); };
    auto kh8w = [&](int f) { return 0.5f * (T(t.kh, i, j, f - 1) + T(t.kh, i, j, f)); };
    auto diffuse = [&](const float* a) {
      auto fx = [&](int q) {
        return -r * kh8u(q) * ((T(a, wrap(q, nx), j, k) - T(a, wrap(q - 1, nx), j, k)) * rdx);
      };
      auto fy = [&](int rr) {
        return -r * kh8v(rr) * ((T(a, i, wrap(rr, ny), k) - T(a, i, wrap(rr - 1, ny), k)) * rdy);
      };
      auto fz = [&](int f) {
        if (f <= 0 || f >= nz) return 0.f;
        return -c.rho_wext[f] * kh8w(f) * ((T(a, i, j, f) - T(a, i, j, f - 1)) * rdz);
      };
      return -((fx(i + 1) - fx(i)) * rdx + (fy(j + 1) - fy(j)) * rdy + (fz(k + 1) - fz(k)) * rdz) * ri;
    };
    o.T[id] = diffuse(s.T);
    o.q[id] = diffuse(s.q);
  }
}

}  // namespace

cudaError_t launch_smag_a(const Dims& d, const Phys& ph, const Cols& c, State in, SmagTau out, cudaStream_t st) {
  dim3 g((d.nx + BX - 1) / BX, (d.ny + BY - 1) / BY, (d.nz + BZ - 1) / BZ);
  k_smag_a<<<g, dim3(BX, BY, BZ), 0, st>>>(d, ph, c, in, out);
  return cudaGetLastError();
}

cudaError_t launch_smag_b(const Dims& d, const Phys& ph, const Cols& c, State in, SmagTau tau, SgsOut out,
                          cudaStream_t st) {
  dim3 g((d.nx + BX - 1) / BX, (d.ny + BY - 1) / BY, (d.nz + 1 + BZ - 1) / BZ);
  k_smag_b<<<g, dim3(BX, BY, BZ), 0, st>>>(d, ph, c, in, tau, out);
  return cudaGetLastError();
}

}  // namespace lexgb
