// lexgb_adjoint.cuh - argument blocks and launchers of the reverse-mode (adjoint) kernels.
#pragma once
#include "lexgb_internal.cuh"

namespace lexgb {

// One acoustic sub-step backwards: from the adjoint of its output (unb .. pnb) to the adjoint of
// its input (ub .. pb), accumulating the adjoints of the stage constants.
struct AcousticVjpArgs {
  const float *p, *trho, *ps;            // input pi', stage theta_rho and pi'_s
  const float *un, *vn, *wn;             // output winds of the sub-step
  const float *unb, *vnb, *wnb, *pnb;    // adjoint of the output
  float *ub, *vb, *wb, *pb;              // adjoint of the input (written)
  float *Rub, *Rvb, *Rwb, *trhob, *psb;  // accumulated
};

// Pointwise part of one stage backwards (after its acoustic loop).
struct StageVjpArgs {
  State xs;                                   // stage input state
  const float* div;                           // its mass divergence
  const float *Tnb, *qnb;                     // adjoint of the stage's theta / qv outputs
  const float *Rub, *Rvb, *Rwb, *trhob, *psb; // from the acoustic loop
  float dts;
  State xsb;                                  // adjoint of the stage input (accumulated)
  State x0b;                                  // adjoint of the big step's input (T, q accumulated)
  const float* acb[4];                        // adjoint of the acoustic loop's input u, v, w, pi' (added to x0b)
  float* cb[5];                               // adjoint of the flux convergence per field (u, v, w, T, q)
  float* divb;                                // adjoint of the mass divergence (written)
  float *sgsb_u, *sgsb_v, *sgsb_w, *sgsb_T, *sgsb_q;  // SGS tendency adjoints (accumulated; null: off)
};

// WENO advection backwards for the five advected fields.
struct AdvVjpArgs {
  State xs;              // stage input (winds for the mass fluxes)
  const float* phi[5];   // advected fields u, v, w, T, q
  const float* cb[5];
  float* P[5][6];        // per-flux stencil adjoints, slot q = point p-3+q of the flux between p-1, p
  float* mb[4];          // mass-flux adjoints: u, v, w fluxes and theta+qv fluxes
  State xsb;             // accumulated
};

// Smagorinsky backwards: forward quantities recomputed at xi0, then the adjoint chain
struct SmagLin {
  float* s[6];   // rho S_11, S_22, S_33, S_12, S_13, S_23
  float* km;     // K_m
  float* kS;     // dK_m / dS^2 (0 where S^2 - N^2/Pr <= 0)
};
struct SmagVjpArgs {
  const float *gu, *gv, *gw, *gT, *gq;  // adjoints of the five SGS tendencies
  float* tb[6];                         // adjoint of tau_ij
  float* khb;                           // adjoint of K_h
  float* sb[6];                         // adjoint of rho S_ij
  float* n2b;                           // adjoint of N^2
  float* kmkb;                          // K_m times its adjoint (optional: the Cs derivative)
  State x0b;                            // accumulated adjoint of the state
};
// out[0] += scale * sum of x[0..n) (FP64 accumulation)
cudaError_t launch_sum_scaled(long long n, const float* x, double scale, double* out, cudaStream_t);
cudaError_t launch_smag_vjp(const Dims&, const Phys&, const Cols&, State x0, const SmagLin&, const SmagVjpArgs&,
                            cudaStream_t);

// win: an L2 access-policy window for the launch (the accumulators)
cudaError_t launch_acoustic_vjp(const Dims&, const Phys&, const Cols&, const AcousticVjpArgs&, float dtau,
                                cudaStream_t, const cudaAccessPolicyWindow* win = nullptr);
cudaError_t launch_stage_pointwise_vjp(const Dims&, const Phys&, const Cols&, const StageVjpArgs&, cudaStream_t);
// x0b (non-null fields): also x0b += xsb, after the update (the first stage's input is the step's input)
cudaError_t launch_massdiv_vjp(const Dims&, const Phys&, const Cols&, const float* divb, State xsb, cudaStream_t,
                               State x0b = State{});
cudaError_t launch_adv_vjp(const Dims&, const Phys&, const Cols&, const AdvVjpArgs&, cudaStream_t);
// y += x over n floats
cudaError_t launch_axpy(float* y, const float* x, size_t n, cudaStream_t);
// y += c over n floats
cudaError_t launch_shift(float* y, float c, size_t n, cudaStream_t);

}  // namespace lexgb
