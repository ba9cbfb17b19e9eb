// lexgb_internal.cuh - device layout, shared reconstruction/physics helpers and kernel
// launchers of the lex_gb300 dynamical core.
//
// Device layout
//   Every field is stored interior-only, x fastest: idx(i, j, k) = (k*ny + j)*nx + i.
//   theta, pi', qv, u, v have nz levels; w has nz+1 levels (faces 0..nz, w = 0 at 0 and nz).
//   u(i) sits on the west face of cell i and v(j) on the south face of cell j; the
//   reference's duplicated periodic face u[nx] (== u[0]) is not stored
//   (padding3u_array, one_step_integration.py:962-972).
//   Lateral halos are periodic and realised by index wrap; the reference's z ghost levels
//   (edge copies, one_step_integration.py:950-959) by clamping.
//   theta is stored as T = theta - theta_ref (theta_ref a constant): every operator on
//   theta is either affine-invariant (WENO reconstructions, flux form + theta*div,
//   gradients) or is rewritten exactly in terms of T, which keeps FP32 increments of a
//   ~300 K field representable.
//
// Base state
//   Horizontally uniform; kept as FP32 per-level columns derived in FP64 on the device
//   (Cols below).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace lexgb {

// namelist_n_constants.py:64-75, evaluated in double and rounded once
constexpr double kRd = 287.04;
constexpr double kRv = 461.5;
constexpr double kCp = 1004.64;
constexpr double kCv = kCp - kRd;
constexpr double kG = 9.80616;
constexpr double kP00 = 100000.0;
constexpr double kReps = kRv / kRd;
constexpr double kRepsm1 = kRv / kRd - 1.0;

constexpr float kWepsMom = 1.0e-16f;    // one_step_integration.py:896
constexpr float kWepsTheta = 1.0e-17f;  // one_step_integration.py:905
constexpr float kWepsQv = 1.0e-18f;     // one_step_integration.py:913
constexpr float kDivDamp = 1.1f;        // one_step_integration.py:546
constexpr double kPrandtl = 1.0 / 3.0;  // turbulence.py:432
constexpr float kInvPrandtl = 3.0f;     // 1 / kPrandtl, exact (x / Pr is x * 3)
constexpr double kCs = 0.18;            // turbulence.py:433
// fmin(1e30, .) of the reference (advection.py:322) would square to inf in FP32; the cap
// below keeps every weight finite.  It only differs from the reference where a ratio
// exceeds 1e18, where the capped weight already dominates the normalised sum.
constexpr float kRatioCap = 1.0e18f;

struct Dims {
  int nx, ny, nz;
  __host__ __device__ __forceinline__ int plane() const { return nx * ny; }
  __host__ __device__ __forceinline__ int at(int i, int j, int k) const { return (k * ny + j) * nx + i; }
  __host__ __device__ __forceinline__ long long cells() const { return (long long)nx * ny * nz; }
  __host__ __device__ __forceinline__ long long faces() const { return (long long)nx * ny * (nz + 1); }
};

// FP32 base-state columns (device pointers into one allocation).
struct Cols {
  const float* rho;       // nz    rho0 at cells
  const float* rho_face;  // nz+1  0.5*(rho0_pad[f] + rho0_pad[f+1]) (ghost levels at the ends)
  const float* rho_face0; // nz+1  same with 0 at f = 0 and f = nz (get_divergence, advection.py:213-215)
  const float* rho_wext;  // nz+1  interpolate_scalar2w(rho0) (pressure_equations.py:123)
  const float* theta0;    // nz
  const float* qv0;       // nz
  const float* trho0;     // nz    theta0*(1+reps*qv0)/(1+qv0)
  const float* d0;        // nz    theta0 - theta_ref
  const float* pi0;       // nz
  const float* dpi0dz;    // nz+1  (pi0_pad[f+1] - pi0_pad[f]) / dz
  const float* rho_inv;   // nz    1 / rho (of the FP32 rho), correctly rounded
  const float* rho_w_inv; // nz+1  1 / (0.5f * (rho[f-1] + rho[f])) on interior faces, 0 at f = 0 and nz
  const float* rho_wext_inv; // nz+1  1 / rho_wext, correctly rounded
};

struct Phys {
  float dx, dy, dz;
  float rdx, rdy, rdz;
  float theta_ref;
  float smag_l2;  // (Cs * cbrt(dx dy dz))^2
  int cor_opt;
  float f_cor;
};

__device__ __forceinline__ int wrap(int i, int n) { return i < 0 ? i + n : (i >= n ? i - n : i); }
__device__ __forceinline__ int clampi(int i, int lo, int hi) { return i < lo ? lo : (i > hi ? hi : i); }

// ---------------------------------------------------------------------------------------------
// reconstruction (advection.py:305-416 and the lateral blocks :424-503)
// ---------------------------------------------------------------------------------------------
// WENO5 value at the face right of c; a..e ordered upwind -> downwind.
// Approximate reciprocal and quotient (PTX rcp.approx / div.approx, flush-to-zero forms, 2 ulp).
// Used in the WENO weights, where every denominator is a normal number (b + eps >= 1e-18, weight
// sums >= 0.1); there the non-ftz forms give the same result but spend extra instructions on the
// subnormal range.
__device__ __forceinline__ float rcp_approx(float x) {
  float r;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}
__device__ __forceinline__ float div_approx(float x, float y) {
  float r;
  asm("div.approx.ftz.f32 %0, %1, %2;" : "=f"(r) : "f"(x), "f"(y));
  return r;
}

__device__ __forceinline__ float weno5(float a, float b, float c, float d, float e, float eps) {
  const float t1 = a - 2.f * b + c, t2 = a - 4.f * b + 3.f * c;
  const float t3 = b - 2.f * c + d, t4 = b - d;
  const float t5 = c - 2.f * d + e, t6 = 3.f * c - 4.f * d + e;
  const float b1 = (13.f / 12.f) * t1 * t1 + 0.25f * t2 * t2;
  const float b2 = (13.f / 12.f) * t3 * t3 + 0.25f * t4 * t4;
  const float b3 = (13.f / 12.f) * t5 * t5 + 0.25f * t6 * t6;
  const float tau = fabsf(b1 - b3);
  const float r1 = fminf(kRatioCap, div_approx(tau, b1 + eps));
  const float r2 = fminf(kRatioCap, div_approx(tau, b2 + eps));
  const float r3 = fminf(kRatioCap, div_approx(tau, b3 + eps));
  const float w1 = 0.1f * (1.f + r1 * r1);
  const float w2 = 0.6f * (1.f + r2 * r2);
  const float w3 = 0.3f * (1.f + r3 * r3);
  const float q1 = (2.f / 6.f) * a + (-7.f / 6.f) * b + (11.f / 6.f) * c;
  const float q2 = (-1.f / 6.f) * b + (5.f / 6.f) * c + (2.f / 6.f) * d;
  const float q3 = (2.f / 6.f) * c + (5.f / 6.f) * d + (-1.f / 6.f) * e;
  return div_approx(w1 * q1 + w2 * q2 + w3 * q3, w1 + w2 + w3);
}

// WENO3 value at the face right of b; a, b, c = s[-1], s[0], s[+1] upwind-ordered.
__device__ __forceinline__ float weno3(float a, float b, float c, float eps) {
  const float b1 = (a - b) * (a - b);
  const float b2 = (b - c) * (b - c);
  const float tau = fabsf(b1 - b2);
  const float r1 = fminf(kRatioCap, div_approx(tau, b1 + eps));
  const float r2 = fminf(kRatioCap, div_approx(tau, b2 + eps));
  const float w1 = (1.f / 3.f) * (1.f + r1 * r1);
  const float w2 = (2.f / 3.f) * (1.f + r2 * r2);
  return div_approx(w1 * (-0.5f * a + 1.5f * b) + w2 * (0.5f * b + 0.5f * c), w1 + w2);
}

// Vertical face value between column entries f-1 and f of an n-entry column s(0..n-1),
// for upward (m >= 0) or downward flow; zero at f = 0 and f = n.  Centred / WENO3 next to
// the ends exactly as vertical_flux_scalar2 / _u2 / _v2 / _w2 do.
template <class F>
__device__ __forceinline__ float vrecon(const F& s, int f, int n, bool up, float eps) {
  if (f <= 0 || f >= n) return 0.f;
  if (up) {
    if (f == 1) return 0.5f * (s(0) + s(1));
    if (f == 2) return weno3(s(0), s(1), s(2), eps);
    if (f == n - 1) return weno3(s(n - 3), s(n - 2), s(n - 1), eps);
    return weno5(s(f - 3), s(f - 2), s(f - 1), s(f), s(f + 1), eps);
  } else {
    if (f == 1) return weno3(s(2), s(1), s(0), eps);
    if (f == n - 1) return 0.5f * (s(n - 1) + s(n - 2));
    if (f == n - 2) return weno3(s(n - 1), s(n - 2), s(n - 3), eps);
    return weno5(s(f + 2), s(f + 1), s(f), s(f - 1), s(f - 2), eps);
  }
}

// jax.lax.select(m >= 0, m*pos, m*neg): ties take the positive branch.
__device__ __forceinline__ float upwind(float m, float pos, float neg) { return m >= 0.f ? m * pos : m * neg; }

// m * (upwind WENO5 value) at the face between s[-1] and s[0], given s[-3..2]: the stencil is
// selected by the sign of the mass flux first, so only one reconstruction is evaluated
// (the reference evaluates both and selects, advection.py:505).
__device__ __forceinline__ float weno_flux(float m, float sm3, float sm2, float sm1, float s0, float sp1, float sp2,
                                           float eps) {
  const bool p = m >= 0.f;
  return m * weno5(p ? sm3 : sp2, p ? sm2 : sp1, p ? sm1 : s0, p ? s0 : sm1, p ? sp1 : sm2, eps);
}

// ---------------------------------------------------------------------------------------------
// two independent reconstructions at once on the packed FP32x2 pipe (sm_100+): each component
// follows weno5 / weno3 above, with the linear weights folded into the candidate polynomials
// (w_k q_k / sum w_k with w_k = d_k (1 + r_k^2)).  Component-wise IEEE round-to-nearest.
// ---------------------------------------------------------------------------------------------
__device__ __forceinline__ float2 f2(float a) { return make_float2(a, a); }
__device__ __forceinline__ float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 sub2(float2 a, float2 b) { return __ffma2_rn(b, f2(-1.f), a); }
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }

__device__ __forceinline__ float2 rcp2(float2 x) { return make_float2(rcp_approx(x.x), rcp_approx(x.y)); }
__device__ __forceinline__ float2 sel2(bool p, float2 a, float2 b) { return p ? a : b; }

__device__ __forceinline__ float2 weno5x2(float2 a, float2 b, float2 c, float2 d, float2 e, float2 eps) {
  const float2 t1 = add2(fma2(b, f2(-2.f), a), c), t2 = fma2(c, f2(3.f), fma2(b, f2(-4.f), a));
  const float2 t3 = add2(fma2(c, f2(-2.f), b), d), t4 = sub2(b, d);
  const float2 t5 = add2(fma2(d, f2(-2.f), c), e), t6 = fma2(d, f2(-4.f), fma2(c, f2(3.f), e));
  const float2 b1 = fma2(mul2(t1, f2(13.f / 12.f)), t1, mul2(mul2(t2, f2(0.25f)), t2));
  const float2 b2 = fma2(mul2(t3, f2(13.f / 12.f)), t3, mul2(mul2(t4, f2(0.25f)), t4));
  const float2 b3 = fma2(mul2(t5, f2(13.f / 12.f)), t5, mul2(mul2(t6, f2(0.25f)), t6));
  const float2 d13 = sub2(b1, b3);
  const float2 tau = make_float2(fabsf(d13.x), fabsf(d13.y));
  float2 r1 = mul2(tau, rcp2(add2(b1, eps))), r2 = mul2(tau, rcp2(add2(b2, eps))), r3 = mul2(tau, rcp2(add2(b3, eps)));
  r1 = make_float2(fminf(kRatioCap, r1.x), fminf(kRatioCap, r1.y));
  r2 = make_float2(fminf(kRatioCap, r2.x), fminf(kRatioCap, r2.y));
  r3 = make_float2(fminf(kRatioCap, r3.x), fminf(kRatioCap, r3.y));
  const float2 s1 = fma2(r1, r1, f2(1.f)), s2 = fma2(r2, r2, f2(1.f)), s3 = fma2(r3, r3, f2(1.f));
  // d_k q_k with d = (0.1, 0.6, 0.3)
  const float2 q1 = fma2(a, f2(0.1f * 2.f / 6.f), fma2(b, f2(0.1f * -7.f / 6.f), mul2(c, f2(0.1f * 11.f / 6.f))));
  const float2 q2 = fma2(b, f2(0.6f * -1.f / 6.f), fma2(c, f2(0.6f * 5.f / 6.f), mul2(d, f2(0.6f * 2.f / 6.f))));
  const float2 q3 = fma2(c, f2(0.3f * 2.f / 6.f), fma2(d, f2(0.3f * 5.f / 6.f), mul2(e, f2(0.3f * -1.f / 6.f))));
  const float2 num = fma2(s1, q1, fma2(s2, q2, mul2(s3, q3)));
  const float2 den = fma2(s1, f2(0.1f), fma2(s2, f2(0.6f), mul2(s3, f2(0.3f))));
  return mul2(num, rcp2(den));
}

__device__ __forceinline__ float2 weno3x2(float2 a, float2 b, float2 c, float2 eps) {
  const float2 dab = sub2(a, b), dbc = sub2(b, c);
  const float2 b1 = mul2(dab, dab), b2 = mul2(dbc, dbc);
  const float2 d12 = sub2(b1, b2);
  const float2 tau = make_float2(fabsf(d12.x), fabsf(d12.y));
  float2 r1 = mul2(tau, rcp2(add2(b1, eps))), r2 = mul2(tau, rcp2(add2(b2, eps)));
  r1 = make_float2(fminf(kRatioCap, r1.x), fminf(kRatioCap, r1.y));
  r2 = make_float2(fminf(kRatioCap, r2.x), fminf(kRatioCap, r2.y));
  const float2 s1 = fma2(r1, r1, f2(1.f)), s2 = fma2(r2, r2, f2(1.f));
  const float2 q1 = fma2(a, f2(-0.5f / 3.f), mul2(b, f2(1.5f / 3.f)));        // (1/3)(-a/2 + 3b/2)
  const float2 q2 = fma2(b, f2(0.5f * 2.f / 3.f), mul2(c, f2(0.5f * 2.f / 3.f)));  // (2/3)(b/2 + c/2)
  const float2 num = fma2(s1, q1, mul2(s2, q2));
  const float2 den = fma2(s1, f2(1.f / 3.f), mul2(s2, f2(2.f / 3.f)));
  return mul2(num, rcp2(den));
}

// m * upwind WENO5 value for two fields sharing the mass flux m (see weno_flux)
__device__ __forceinline__ float2 weno_flux_x2(float m, float2 sm3, float2 sm2, float2 sm1, float2 s0, float2 sp1,
                                               float2 sp2, float2 eps) {
  const bool p = m >= 0.f;
  return mul2(f2(m), weno5x2(sel2(p, sm3, sp2), sel2(p, sm2, sp1), sel2(p, sm1, s0), sel2(p, s0, sm1),
                             sel2(p, sp1, sm2), eps));
}

// m * (upwind vertical face value) at face f of an n-entry column (see vrecon); zero at the ends.
template <class F>
__device__ __forceinline__ float vflux(float m, const F& s, int f, int n, float eps) {
  if (f <= 0 || f >= n) return 0.f;
  const bool up = m >= 0.f;
  if (f >= 3 && f <= n - 3)
    return m * weno5(up ? s(f - 3) : s(f + 2), up ? s(f - 2) : s(f + 1), up ? s(f - 1) : s(f), up ? s(f) : s(f - 1),
                     up ? s(f + 1) : s(f - 2), eps);
  return m * vrecon(s, f, n, up, eps);
}

// ---------------------------------------------------------------------------------------------
// thermodynamics
// ---------------------------------------------------------------------------------------------
// density potential temperature theta*(1+reps*qv)/(1+qv) (one_step_integration.py:269)
__device__ __forceinline__ float theta_rho(float T, float q, float theta_ref) {
  return (theta_ref + T) * (1.f + (float)kReps * q) / (1.f + q);
}

// g*(theta_rho - theta_rho0)/theta_rho0 (pressure_equations.py:162-172), with
// theta_rho - theta_rho0 = [theta0 (reps-1)(q - q0) + (theta - theta0)(1 + reps q)(1 + q0)] / ((1+q)(1+q0))
// evaluated from T = theta - theta_ref and d0 = theta0 - theta_ref.
__device__ __forceinline__ float buoyancy_at(float T, float q, int k, const Cols& c) {
  const float th0 = c.theta0[k], q0 = c.qv0[k];
  const float num = th0 * (float)(kReps - 1.0) * (q - q0) + (T - c.d0[k]) * (1.f + (float)kReps * q) * (1.f + q0);
  return (float)kG * (num / ((1.f + q) * (1.f + q0))) / c.trho0[k];
}

// ---------------------------------------------------------------------------------------------
// kernel launchers (stream-ordered; return cudaGetLastError())
// ---------------------------------------------------------------------------------------------
struct State {
  float* T;   // theta - theta_ref
  float* u;
  float* v;
  float* w;   // nz+1 levels
  float* p;   // pi'
  float* q;   // qv
};

struct SlowOut {
  float* Ru;
  float* Rv;
  float* Rw;
  float* T_next;
  float* q_next;
  float* dT;   // optional: d_theta_dt record (adv + sgs)
  float* dq;   // optional
};

struct Sgs {
  const float* u;
  const float* v;
  const float* w;
  const float* T;
  const float* q;
};

cudaError_t launch_div_trho(const Dims&, const Phys&, const Cols&, State in, float* div, float* trho, cudaStream_t);
// div_out / trho_out: when given, the divergence div(rho0 u) and theta_rho of `in` are computed here
// (inside the vertical-march kernel where it runs, else by launch_div_trho first) and `div` is unused
cudaError_t launch_adv_scalars(const Dims&, const Phys&, const Cols&, State in, const float* div, const float* T0,
                               const float* q0, Sgs sgs, float dts, SlowOut out, cudaStream_t,
                               float* div_out = nullptr, float* trho_out = nullptr);
// once per process, before the first launch (opts the momentum kernel into > 48 KB of shared memory)
cudaError_t init_weno_attributes();
// u, v, w together; wmode 0: R_w = adv_w + b8w + sgs_w; 1: adv_w only; 2: b8w only
cudaError_t launch_adv_momentum(const Dims&, const Phys&, const Cols&, State in, const float* div, Sgs sgs, float* Ru,
                                float* Rv, float* Rw, int wmode, cudaStream_t);
struct AcousticIn {
  const float *u, *v, *w, *p;       // sub-step start
  const float *Ru, *Rv, *Rw;        // slow tendencies
  const float *trho;                // density potential temperature of the stage state
  const float *ps;                  // pi' of the stage state (pip_star)
};
struct AcousticOut { float *u, *v, *w, *p; };
// rev: walk the grid in reversed block order; win: an L2 access-policy window for the launch
cudaError_t launch_acoustic(const Dims&, const Phys&, const Cols&, AcousticIn in, AcousticOut out, float dtau,
                            cudaStream_t, int rev = 0, const cudaAccessPolicyWindow* win = nullptr);
// two sub-steps in one launch (temporal blocking); in and out must not alias
cudaError_t launch_acoustic_pair(const Dims&, const Phys&, const Cols&, AcousticIn in, AcousticOut out, float dtau,
                                 cudaStream_t);
cudaError_t init_acoustic_attributes();
// All sub-steps of one stage in one cooperative launch (nsub >= 2): each block keeps its tile of pi'
// in shared memory; u, v and w of sub-step s are read from u[src] and written to u[dst] with
// src = 0 (the stage's input winds, read only) for s = 0, else 1 + ((s-1) & 1), and dst = 3 (the
// stage's output winds) for the last sub-step, else 1 + (s & 1); hb[0]/hb[1] (field-sized) carry the
// tiles' edge pi' between sub-steps.  The stage's input winds and pi' may alias its outputs.
// bar: one word, zeroed by the launcher; status: the context's sticky status word
// (LEXGB_ERR_TIMEOUT when a bounded wait gave up after spin_limit polls).
struct PersistIO {
  float *u[4], *v[4], *w[4];
  const float* p0;
  float* po;
  const float *Ru, *Rv, *Rw, *trho, *ps;
  float* hb[2];
  unsigned* bar;
  int* status;
  long long spin_limit;
  int unreachable;   // test mode: every grid-barrier wait expects one arrival too many and gives up
  int nsub;
  float dtau;
};
// one sub-step on 32 x 4 x 8 blocks sharing values between warps (needs nx % 32 == 0, ny % 4 == 0);
// same results as launch_acoustic
bool acoustic_tile_fits(const Dims&);
cudaError_t launch_acoustic_tile(const Dims&, const Phys&, const Cols&, AcousticIn in, AcousticOut out, float dtau,
                                 cudaStream_t, int rev = 0, const cudaAccessPolicyWindow* win = nullptr);
// blocks of the persistent kernel for this grid, or 0 when the grid does not fit it
int acoustic_persist_blocks(const Dims&);
size_t acoustic_persist_smem(const Dims&);
cudaError_t launch_acoustic_persist(const Dims&, const Phys&, const Cols&, const PersistIO&, cudaStream_t,
                                    const cudaAccessPolicyWindow* win = nullptr);
// diagnostics of the acoustic operators on one state
cudaError_t launch_diag_pgf(const Dims&, const Phys&, const Cols&, const float* p, const float* trho, float* pu,
                            float* pv, float* pw, cudaStream_t);
cudaError_t launch_diag_advpi(const Dims&, const Phys&, const Cols&, const float* ps, const float* u,
                              const float* v, const float* w, float* out, cudaStream_t);
// Smagorinsky: stage A writes tau11, tau22, tau33, tau12, tau13, tau23, kh (+ optional n2, km)
struct SmagTau { float *t11, *t22, *t33, *t12, *t13, *t23, *kh, *n2, *km; };
cudaError_t launch_smag_a(const Dims&, const Phys&, const Cols&, State in, SmagTau out, cudaStream_t);
struct SgsOut { float *u, *v, *w, *T, *q; };
cudaError_t launch_smag_b(const Dims&, const Phys&, const Cols&, State in, SmagTau tau, SgsOut out, cudaStream_t);

// learned SGS correction: network input from the state (16 BF16 channels a cell) and the
// correction (8 FP32 channels a cell, 5 used) scaled and added back to the state
cudaError_t launch_sgs_pack(int nx, int ny, int nz, const float* T, const float* u, const float* v, const float* w,
                            const float* q, float theta_ref, const float* lo, const float* rin, void* x16,
                            cudaStream_t);
cudaError_t conv_prepare();  // one-time set-up of the CNN convolution kernels (outside graph capture)
// one convolution (cin 16 or 32, cout 8, 16 or 32); pdl: launched as a programmatic dependent of
// the previous kernel of the stream, which must not write w or bias
cudaError_t launch_cnn_conv3d(int nx, int ny, int nz, int cin, int cout, const void* x, const void* w,
                              const float* bias, float* pre, void* ybf, float* yf, int gelu, int creal,
                              cudaStream_t st, bool pdl);
cudaError_t launch_sgs_unpack(int nx, int ny, int nz, const float* corr, const float* rout, float* T, float* u,
                              float* v, float* w, float* q, cudaStream_t, bool pdl);

// layout conversion between the reference's padded [x][y][z] host layout and the device layout
// kind: 0 scalar, 1 u, 2 v, 3 w
cudaError_t launch_import_padded(const Dims&, const void* src, int src_f64, int kind, double offset, float* dst,
                                 cudaStream_t);
cudaError_t launch_export_padded(const Dims&, const float* src, int kind, double offset, void* dst, int dst_f64,
                                 cudaStream_t);
// interior export in reference C order (x slowest, z fastest); u/v with the duplicated face
cudaError_t launch_export_interior(const Dims&, const float* src, int kind, double offset, double* dst, cudaStream_t);

// FP64 base state
cudaError_t launch_hydrostatic(int nz, double dz, const double* theta0, const double* qv0, double* pi0,
                               double* rho0, cudaStream_t);
constexpr int kColumnRows = 13;   // rows of nz + 2 floats in the column table (the Cols fields, in order)
cudaError_t launch_build_columns(int nz, double dz, double theta_ref, const double* theta0, const double* qv0,
                                 const double* pi0, const double* rho0, float* table, cudaStream_t);
// FP64 budgets: partial sums per block into `partial` (nblocks x 4), then a final pass into out[4]
int budget_blocks(const Dims&);
constexpr int kBudgetSums = 5;   // mass, vapour, kinetic energy, rho0 theta, total energy
cudaError_t launch_budget(const Dims&, const Phys&, const Cols&, State in, const double* rho0_col,
                          const double* pi0_col, double theta_ref, double* partial, double* out, cudaStream_t);
cudaError_t launch_count_nonfinite(const float* a, long long n, unsigned long long* count, cudaStream_t);

}  // namespace lexgb
