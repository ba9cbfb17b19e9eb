// capi.cu - the C ABI of include/lexgb.h: context, device buffers, the Wicker-Skamarock RK3
// stage driver (one_sprint_functions.py:10-30, one_step_integration.py:16-447), CUDA-graph
// replay of a big step, host transfers, operator diagnostics and FP64 budgets.
#include <cuda_runtime.h>
#include <math.h>
#include <nvtx3/nvToolsExt.h>
#include <stdio.h>
#include <string.h>

#include <string>
#include <utility>
#include <vector>

#include "../../include/lexgb.h"
#include "lexgb_adjoint.cuh"

namespace {
// NVTX range over an ABI call (no cost without a profiler attached)
struct NvtxRange {
  explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
  ~NvtxRange() { nvtxRangePop(); }
};
}  // namespace

using namespace lexgb;

namespace {

thread_local std::string g_last_error;

int fail(int code, const std::string& msg) {
  g_last_error = msg;
  return code;
}

#define CK(call)                                                                                  \
  do {                                                                                            \
    cudaError_t e_ = (call);                                                                      \
    if (e_ != cudaSuccess)                                                                        \
      return fail(LEXGB_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_));            \
  } while (0)

#define CKS(call)                                                                                 \
  do {                                                                                            \
    int s_ = (call);                                                                              \
    if (s_ != LEXGB_OK) return s_;                                                                \
  } while (0)

constexpr int NFIELD = 6;  // T u v w p q

}  // namespace

namespace lexgb {
// lets other translation units of the library report through lexgb_last_error
void record_error(const std::string& msg) { g_last_error = msg; }
}  // namespace lexgb

struct lexgb_ctx {
  lexgb_config cfg{};
  Dims d{};
  Phys ph{};
  double theta_ref = 0.0;
  cudaStream_t stream = nullptr;
  cudaStream_t own_stream = nullptr;
  // host <-> device copies of the state: a copy stream beside the compute stream, one event per
  // field, so that a field's copy overlaps the previous field's layout conversion
  cudaStream_t copy_stream = nullptr;
  cudaEvent_t field_ev[NFIELD] = {};
  size_t fstride = 0;  // floats per field allocation (nx*ny*(nz+1))
  // FP64 padded base columns theta0 | qv0 | pi0 | rho0 and the FP32 table
  double* base64 = nullptr;
  float* tab = nullptr;
  Cols cols{};
  bool base_set = false;
  bool state_set = false;
  // field arena
  float* arena = nullptr;
  size_t arena_fields = 0;
  State A{}, B{}, C{};
  float *Xu, *Xv, *Xw, *Xp, *Yu, *Yv, *Yw, *Yp;
  float *Ru, *Rv, *Rw, *trho, *div;
  float* sgs[5];
  float* tau[7];
  float* diag[3];
  // record mode (allocated on first use)
  float* rec_arena = nullptr;
  State S[3]{}, R0{};
  float* recdT[3]{};
  float* recdq[3]{};
  bool recorded = false;
  // staging
  void* stage = nullptr;
  size_t stage_bytes = 0;
  double* partial = nullptr;
  double* budget = nullptr;
  unsigned long long* count = nullptr;
  // reverse mode: workspace of the recomputed step and the adjoint fields (allocated on first use)
  float* adj_arena = nullptr;
  bool adj_kept = false;  // the workspace holds a step kept by lexgb_step_keep
  // learned SGS correction (allocated on first use): weights, biases, ranges, activations
  char* sgs_arena = nullptr;
  bool sgs_on = false;
  void* sgs_w[4]{};
  float* sgs_b[4]{};
  float *sgs_lo = nullptr, *sgs_rin = nullptr, *sgs_rout = nullptr, *sgs_corr = nullptr;
  void *sgs_x = nullptr, *sgs_a0 = nullptr, *sgs_a1 = nullptr;
  // Smagorinsky constant and the FP64 accumulator of d(seed . output)/dCs
  double cs = kCs;
  double* cs_bar = nullptr;
  // persisting L2 window over R_u, R_v, R_w, theta_rho for the acoustic sub-steps
  cudaAccessPolicyWindow l2win{};
  bool l2on = false;
  // persistent acoustic kernel: blocks (0: not used for this grid), its barrier word and the
  // sticky device status word (LEXGB_ERR_TIMEOUT after a grid-barrier wait gave up)
  int persist_blocks = 0;
  int ak = LEXGB_ACOUSTIC_ROWS;   // the resolved acoustic form
  unsigned* sync = nullptr;   // [0] barrier arrivals, [1] status
  long long spin_limit = 1LL << 24;
  int barrier_test = 0;   // lexgb_set_barrier_limit with polls < 0
  // graph of one big step
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t gexec = nullptr;
};

namespace {

State fields_at(float* base, size_t stride) {
  State s;
  s.T = base + 0 * stride;
  s.u = base + 1 * stride;
  s.v = base + 2 * stride;
  s.w = base + 3 * stride;
  s.p = base + 4 * stride;
  s.q = base + 5 * stride;
  return s;
}

float* field_of(const State& s, int f) {
  switch (f) {
    case 0: return s.T;
    case 1: return s.u;
    case 2: return s.v;
    case 3: return s.w;
    case 4: return s.p;
    default: return s.q;
  }
}

int kind_of(int f) { return f == 1 ? 1 : (f == 2 ? 2 : (f == 3 ? 3 : 0)); }

size_t padded_count(const Dims& d, int kind) {
  return (size_t)(d.nx + 6 + (kind == 1)) * (d.ny + 6 + (kind == 2)) * (d.nz + 2 + (kind == 3));
}

size_t interior_count(const Dims& d, int kind) {
  return (size_t)(d.nx + (kind == 1)) * (d.ny + (kind == 2)) * (d.nz + (kind == 3));
}

struct StagePlan {
  double dts[3];
  int n[3];
  double dtau[3];
};

// one_sprint_functions.py:19-21 and one_step_integration.py:121-122, :253-254
StagePlan plan_of(const lexgb_config& c) {
  StagePlan p;
  const double dt_sound = c.dt / c.n_sound;
  p.dts[0] = c.dt / 3.0;
  p.dts[1] = c.dt / 2.0;
  p.dts[2] = c.dt;
  p.n[0] = 1;
  p.dtau[0] = p.dts[0];
  p.n[1] = (int)lround(p.dts[1] / dt_sound);
  p.n[2] = (int)lround(p.dts[2] / dt_sound);
  p.dtau[1] = p.dtau[2] = dt_sound;
  return p;
}

// one acoustic sub-step with the context's per-sub-step kernel (both give identical results)
cudaError_t sub_step(lexgb_ctx* c, const AcousticIn& in, const AcousticOut& out, float dtau, int rev,
                     const cudaAccessPolicyWindow* win) {
  if (c->ak == LEXGB_ACOUSTIC_TILE) return launch_acoustic_tile(c->d, c->ph, c->cols, in, out, dtau, c->stream, rev, win);
  return launch_acoustic(c->d, c->ph, c->cols, in, out, dtau, c->stream, rev, win);
}

int run_smag(lexgb_ctx* c, const State& x, float* n2, float* km) {
  SmagTau t{c->tau[0], c->tau[1], c->tau[2], c->tau[3], c->tau[4], c->tau[5], c->tau[6], n2, km};
  CK(launch_smag_a(c->d, c->ph, c->cols, x, t, c->stream));
  SgsOut o{c->sgs[0], c->sgs[1], c->sgs[2], c->sgs[3], c->sgs[4]};
  CK(launch_smag_b(c->d, c->ph, c->cols, x, t, o, c->stream));
  return LEXGB_OK;
}

// One WS-RK3 stage: xi_out = xi0 + dts * F(xis) (rk_sub_step0/1/2 with solver_opt = 2).
int run_stage(lexgb_ctx* c, int s, const State& xi0, const State& xis, const State& out, float* dT, float* dq) {
  const StagePlan p = plan_of(c->cfg);
  const bool sgs_on = c->cfg.turb_opt == 1;
  Sgs sg{nullptr, nullptr, nullptr, nullptr, nullptr};
  if (sgs_on) sg = Sgs{c->sgs[0], c->sgs[1], c->sgs[2], c->sgs[3], c->sgs[4]};
  SlowOut so{nullptr, nullptr, nullptr, out.T, out.q, dT, dq};
  // theta/qv advection, which also forms div(rho0 u) and theta_rho of the stage state
  CK(launch_adv_scalars(c->d, c->ph, c->cols, xis, nullptr, xi0.T, xi0.q, sg, (float)p.dts[s], so, c->stream,
                        c->div, c->trho));
  CK(launch_adv_momentum(c->d, c->ph, c->cols, xis, c->div, sg, c->Ru, c->Rv, c->Rw, 0, c->stream));
  // acoustic sub-steps from xi0's winds and pi'; pi'_s is the stage state's pi'.  With
  // acoustic_pairs, sub-steps go two per launch (an odd count starts with a single one).
  const int n = p.n[s];
  const float dtau = (float)p.dtau[s];
  // (pi'_s stays outside the persisting window: a fifth field there, 71 MB at 192x192x96, measured
  // 2.74 ms per step against 2.70 ms with four, the set-aside crowding out the moving state)
  const float* ps = xis.p;
  AcousticIn in{xi0.u, xi0.v, xi0.w, xi0.p, c->Ru, c->Rv, c->Rw, c->trho, ps};
  const AcousticOut X{c->Xu, c->Xv, c->Xw, c->Xp}, Y{c->Yu, c->Yv, c->Yw, c->Yp};
  const AcousticOut O{out.u, out.v, out.w, out.p};
  if (c->persist_blocks > 0 && n >= 2) {  // all sub-steps in one persistent launch (in and out may alias)
    PersistIO io{};
    io.u[0] = xi0.u; io.u[1] = c->Xu; io.u[2] = c->Yu; io.u[3] = out.u;
    io.v[0] = xi0.v; io.v[1] = c->Xv; io.v[2] = c->Yv; io.v[3] = out.v;
    io.w[0] = xi0.w; io.w[1] = c->Xw; io.w[2] = c->Yw; io.w[3] = out.w;
    io.p0 = xi0.p; io.po = out.p;
    io.Ru = c->Ru; io.Rv = c->Rv; io.Rw = c->Rw; io.trho = c->trho; io.ps = ps;
    io.hb[0] = c->Xp; io.hb[1] = c->Yp;
    io.bar = c->sync;
    io.status = reinterpret_cast<int*>(c->sync + 1);
    io.spin_limit = c->spin_limit;
    io.unreachable = c->barrier_test;
    io.nsub = n;
    io.dtau = dtau;
    CK(launch_acoustic_persist(c->d, c->ph, c->cols, io, c->stream, c->l2on ? &c->l2win : nullptr));
    return LEXGB_OK;
  }
  const bool pairs = c->cfg.acoustic_pairs != 0 && c->d.nx % 4 == 0;  // the pair kernel needs nx % 4 == 0
  const int nsingle = pairs ? (n & 1) : n;
  const int launches = nsingle + (pairs ? n / 2 : 0);
  const bool alias = (out.u == xi0.u);
  for (int l = 1; l <= launches; ++l) {
    AcousticOut tgt = (l == launches && !(alias && launches == 1)) ? O : ((l & 1) ? X : Y);
    if (l <= nsingle)
      CK(sub_step(c, in, tgt, dtau, l & 1, c->l2on ? &c->l2win : nullptr));
    else
      CK(launch_acoustic_pair(c->d, c->ph, c->cols, in, tgt, dtau, c->stream));
    in.u = tgt.u;
    in.v = tgt.v;
    in.w = tgt.w;
    in.p = tgt.p;
  }
  if (alias && launches == 1) {  // one launch into the buffer it started from: staged through X
    const size_t bytes = c->fstride * sizeof(float);
    CK(cudaMemcpyAsync(out.u, c->Xu, bytes, cudaMemcpyDeviceToDevice, c->stream));
    CK(cudaMemcpyAsync(out.v, c->Xv, bytes, cudaMemcpyDeviceToDevice, c->stream));
    CK(cudaMemcpyAsync(out.w, c->Xw, bytes, cudaMemcpyDeviceToDevice, c->stream));
    CK(cudaMemcpyAsync(out.p, c->Xp, bytes, cudaMemcpyDeviceToDevice, c->stream));
  }
  return LEXGB_OK;
}

// One big step A -> A (stage 0: A -> B, stage 1: B -> C, stage 2: C -> A in place).
int run_step(lexgb_ctx* c) {
  if (c->cfg.turb_opt == 1) CKS(run_smag(c, c->A, nullptr, nullptr));
  CKS(run_stage(c, 0, c->A, c->A, c->B, nullptr, nullptr));
  CKS(run_stage(c, 1, c->A, c->B, c->C, nullptr, nullptr));
  CKS(run_stage(c, 2, c->A, c->C, c->A, nullptr, nullptr));
  return LEXGB_OK;
}

// the learned SGS correction of the state in A: pack, four convolutions, unpack
constexpr int SGS_CIN[4] = {16, 32, 32, 32}, SGS_COUT[4] = {32, 32, 32, 8};

int run_sgs(lexgb_ctx* c) {
  const Dims& d = c->d;
  // programmatic dependent launches only on a created stream (the step graph is captured on the
  // context's own stream); on the legacy or per-thread default stream, plain stream order
  const bool pdl = c->stream != nullptr && c->stream != cudaStreamLegacy && c->stream != cudaStreamPerThread;
  CK(launch_sgs_pack(d.nx, d.ny, d.nz, c->A.T, c->A.u, c->A.v, c->A.w, c->A.q, (float)c->theta_ref, c->sgs_lo,
                     c->sgs_rin, c->sgs_x, c->stream));
  const void* in[4] = {c->sgs_x, c->sgs_a0, c->sgs_a1, c->sgs_a0};
  void* out[3] = {c->sgs_a0, c->sgs_a1, c->sgs_a0};
  for (int l = 0; l < 4; ++l) {
    const bool last = l == 3;
    // programmatic dependents: the weights and biases are the context's copies, written only by
    // lexgb_set_sgs_net, so each layer stages them while the previous kernel finishes
    CK(launch_cnn_conv3d(d.nx, d.ny, d.nz, SGS_CIN[l], SGS_COUT[l], in[l], c->sgs_w[l], c->sgs_b[l], nullptr,
                         last ? nullptr : out[l], last ? c->sgs_corr : nullptr, last ? 0 : 1, last ? 5 : SGS_COUT[l],
                         c->stream, pdl));
  }
  CK(launch_sgs_unpack(d.nx, d.ny, d.nz, c->sgs_corr, c->sgs_rout, c->A.T, c->A.u, c->A.v, c->A.w, c->A.q,
                       c->stream, pdl));
  return LEXGB_OK;
}

int run_big_step(lexgb_ctx* c) {
  CKS(run_step(c));
  if (c->sgs_on) CKS(run_sgs(c));
  return LEXGB_OK;
}

int ensure_record(lexgb_ctx* c) {
  if (c->rec_arena) return LEXGB_OK;
  const size_t nf = 4 * NFIELD + 6;
  cudaError_t e = cudaMalloc(&c->rec_arena, nf * c->fstride * sizeof(float));
  if (e != cudaSuccess) return fail(LEXGB_ERR_ALLOC, std::string("record buffers: ") + cudaGetErrorString(e));
  for (int s = 0; s < 3; ++s) c->S[s] = fields_at(c->rec_arena + (size_t)s * NFIELD * c->fstride, c->fstride);
  c->R0 = fields_at(c->rec_arena + (size_t)3 * NFIELD * c->fstride, c->fstride);
  float* t = c->rec_arena + (size_t)4 * NFIELD * c->fstride;
  for (int s = 0; s < 3; ++s) {
    c->recdT[s] = t + (size_t)(2 * s) * c->fstride;
    c->recdq[s] = t + (size_t)(2 * s + 1) * c->fstride;
  }
  return LEXGB_OK;
}

int copy_state(lexgb_ctx* c, const State& dst, const State& src) {
  for (int f = 0; f < NFIELD; ++f)
    CK(cudaMemcpyAsync(field_of(dst, f), field_of(src, f), c->fstride * sizeof(float), cudaMemcpyDeviceToDevice,
                       c->stream));
  return LEXGB_OK;
}

int check_ready(lexgb_ctx* c) {
  if (!c) return fail(LEXGB_ERR_ARG, "null context");
  if (!c->base_set) return fail(LEXGB_ERR_STATE, "base state not set (lexgb_set_base_columns / lexgb_integrate_base_state)");
  if (!c->state_set) return fail(LEXGB_ERR_STATE, "prognostic state not uploaded (lexgb_upload_state)");
  return LEXGB_OK;
}

// The device status word (after the stream is idle): LEXGB_ERR_TIMEOUT once when a bounded wait of the
// persistent acoustic kernel gave up, and the word is cleared.
int take_status(lexgb_ctx* c) {
  if (!c->sync) return LEXGB_OK;
  int st = 0;
  CK(cudaMemcpyAsync(&st, c->sync + 1, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  if (st == 0) return LEXGB_OK;
  CK(cudaMemsetAsync(c->sync + 1, 0, sizeof(int), c->stream));
  CK(cudaStreamSynchronize(c->stream));
  return fail(LEXGB_ERR_TIMEOUT, "a grid-barrier wait of the persistent acoustic kernel gave up; the state is "
                                 "invalid (upload it again)");
}

int ensure_stage(lexgb_ctx* c, size_t bytes) {
  if (c->stage_bytes >= bytes) return LEXGB_OK;
  if (c->stage) cudaFree(c->stage);
  c->stage = nullptr;
  c->stage_bytes = 0;
  cudaError_t e = cudaMalloc(&c->stage, bytes);
  if (e != cudaSuccess) return fail(LEXGB_ERR_ALLOC, std::string("staging buffer: ") + cudaGetErrorString(e));
  c->stage_bytes = bytes;
  return LEXGB_OK;
}

void drop_graph(lexgb_ctx* c) {
  if (c->gexec) cudaGraphExecDestroy(c->gexec);
  if (c->graph) cudaGraphDestroy(c->graph);
  c->gexec = nullptr;
  c->graph = nullptr;
}

int build_table(lexgb_ctx* c) {
  const int nz = c->d.nz;
  double th1 = 0.0;
  CK(cudaMemcpyAsync(&th1, c->base64 + 1, sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  c->theta_ref = c->cfg.theta_ref != 0.0 ? c->cfg.theta_ref : th1;
  c->ph.theta_ref = (float)c->theta_ref;
  if ((double)c->ph.theta_ref != c->theta_ref)
    return fail(LEXGB_ERR_ARG, "theta_ref must be exactly representable in FP32");
  const size_t S = nz + 2;
  CK(launch_build_columns(nz, c->cfg.dz, c->theta_ref, c->base64, c->base64 + S, c->base64 + 2 * S,
                          c->base64 + 3 * S, c->tab, c->stream));
  float* t = c->tab;
  c->cols = Cols{t,         t + S,     t + 2 * S, t + 3 * S, t + 4 * S,  t + 5 * S,
                 t + 6 * S, t + 7 * S, t + 8 * S, t + 9 * S, t + 10 * S, t + 11 * S, t + 12 * S};
  c->base_set = true;
  c->adj_kept = false;
  drop_graph(c);
  return LEXGB_OK;
}

}  // namespace

extern "C" {

// The acoustic sub-steps of a stage all read R_u, R_v, R_w and theta_rho (four adjacent arena
// fields): a persisting L2 window over them (up to the device's set-aside maximum) keeps them
// on chip across the 16 or 32 sub-steps, so only the moving state streams through HBM.  The
// set-aside is a limit of this process's context; failures leave normal caching.
static void setup_l2_window(lexgb_ctx* c) {
  int dev = 0, max_persist = 0, max_window = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&max_persist, cudaDevAttrMaxPersistingL2CacheSize, dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&max_window, cudaDevAttrMaxAccessPolicyWindowSize, dev) != cudaSuccess ||
      max_persist <= 0 || max_window <= 0) {
    cudaGetLastError();
    return;
  }
  size_t bytes = 4 * c->fstride * sizeof(float);   // R_u, R_v, R_w, theta_rho
  if (bytes > (size_t)max_window) bytes = (size_t)max_window;
  size_t setaside = bytes < (size_t)max_persist ? bytes : (size_t)max_persist;
  size_t cur = 0;
  if (cudaDeviceGetLimit(&cur, cudaLimitPersistingL2CacheSize) != cudaSuccess) cur = 0;
  if (cur < setaside && cudaDeviceSetLimit(cudaLimitPersistingL2CacheSize, setaside) != cudaSuccess) {
    cudaGetLastError();
    return;
  }
  if (cur > setaside) setaside = cur;
  c->l2win.base_ptr = c->Ru;
  c->l2win.num_bytes = bytes;
  c->l2win.hitRatio = setaside >= bytes ? 1.0f : (float)setaside / (float)bytes;
  c->l2win.hitProp = cudaAccessPropertyPersisting;
  c->l2win.missProp = cudaAccessPropertyStreaming;
  c->l2on = true;
}

int lexgb_default_config(lexgb_config* cfg) {
  if (!cfg) return fail(LEXGB_ERR_ARG, "null config");
  memset(cfg, 0, sizeof(*cfg));
  cfg->nx = 240;  // namelist_n_constants.py:20-22
  cfg->ny = 240;
  cfg->nz = 120;
  cfg->dx = cfg->dy = cfg->dz = 100.0;
  cfg->dt = 1.0;
  cfg->n_sound = 32;
  cfg->turb_opt = 0;
  cfg->cor_opt = 0;
  cfg->f_cor = 1.0e-4;
  cfg->theta_ref = 0.0;
  cfg->acoustic_pairs = 0;
  return LEXGB_OK;
}

int lexgb_create(const lexgb_config* cfg, lexgb_ctx** out) {
  if (!cfg || !out) return fail(LEXGB_ERR_ARG, "null argument");
  *out = nullptr;
  if (cfg->nx < 4 || cfg->ny < 4 || cfg->nz < 6)
    return fail(LEXGB_ERR_ARG, "grid too small: need nx, ny >= 4 and nz >= 6");
  if ((long long)cfg->nx * cfg->ny * (cfg->nz + 1) >= (1LL << 31))
    return fail(LEXGB_ERR_ARG, "grid too large: nx*ny*(nz+1) must be < 2^31");
  if (!(cfg->dx > 0) || !(cfg->dy > 0) || !(cfg->dz > 0) || !(cfg->dt > 0))
    return fail(LEXGB_ERR_ARG, "dx, dy, dz and dt must be positive");
  if (cfg->n_sound < 1) return fail(LEXGB_ERR_ARG, "n_sound must be >= 1");
  if (cfg->turb_opt != 0 && cfg->turb_opt != 1)
    return fail(LEXGB_ERR_ARG, "turb_opt must be 0 or 1 (the anisotropic turb_opt=2 is not provided)");
  if (cfg->cor_opt < 0 || cfg->cor_opt > 2) return fail(LEXGB_ERR_ARG, "cor_opt must be 0, 1 or 2");
  if (!(cfg->cs >= 0.0)) return fail(LEXGB_ERR_ARG, "cs must be >= 0 (0: the default 0.18)");
  if (cfg->acoustic_pairs != 0 && cfg->acoustic_pairs != 1) return fail(LEXGB_ERR_ARG, "acoustic_pairs must be 0 or 1");
  if (cfg->acoustic_kernel < LEXGB_ACOUSTIC_AUTO || cfg->acoustic_kernel > LEXGB_ACOUSTIC_PERSISTENT)
    return fail(LEXGB_ERR_ARG, "acoustic_kernel must be LEXGB_ACOUSTIC_AUTO, _ROWS, _TILE or _PERSISTENT");
  lexgb_ctx* c = new lexgb_ctx();
  c->cfg = *cfg;
  c->d = Dims{cfg->nx, cfg->ny, cfg->nz};
  c->ph.dx = (float)cfg->dx;
  c->ph.dy = (float)cfg->dy;
  c->ph.dz = (float)cfg->dz;
  c->ph.rdx = (float)(1.0 / cfg->dx);
  c->ph.rdy = (float)(1.0 / cfg->dy);
  c->ph.rdz = (float)(1.0 / cfg->dz);
  c->cs = cfg->cs > 0.0 ? cfg->cs : kCs;
  const double l = c->cs * cbrt(cfg->dx * cfg->dy * cfg->dz);
  c->ph.smag_l2 = (float)(l * l);
  c->ph.cor_opt = cfg->cor_opt;
  c->ph.f_cor = (float)cfg->f_cor;
  c->fstride = (size_t)cfg->nx * cfg->ny * (cfg->nz + 1);
  c->fstride = (c->fstride + 63) / 64 * 64;  // 256-byte aligned fields
  auto bail = [&](int code, const std::string& m) {
    lexgb_destroy(c);
    return fail(code, m);
  };
  cudaError_t e = cudaStreamCreateWithFlags(&c->own_stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->copy_stream, cudaStreamNonBlocking);
  for (int f = 0; f < NFIELD && e == cudaSuccess; ++f) e = cudaEventCreateWithFlags(&c->field_ev[f], cudaEventDisableTiming);
  if (e != cudaSuccess) return bail(LEXGB_ERR_CUDA, std::string("stream: ") + cudaGetErrorString(e));
  e = init_weno_attributes();
  if (e == cudaSuccess) e = init_acoustic_attributes();
  if (e != cudaSuccess) return bail(LEXGB_ERR_CUDA, std::string("kernel attributes: ") + cudaGetErrorString(e));
  c->stream = c->own_stream;
  // 3 states + 2 acoustic ping-pong sets + R(3) + trho + div + sgs(5) + tau(7) + diag(3)
  c->arena_fields = 3 * NFIELD + 8 + 5 + 5 + 7 + 3;
  e = cudaMalloc(&c->arena, c->arena_fields * c->fstride * sizeof(float));
  if (e != cudaSuccess) return bail(LEXGB_ERR_ALLOC, std::string("field arena: ") + cudaGetErrorString(e));
  e = cudaMemsetAsync(c->arena, 0, c->arena_fields * c->fstride * sizeof(float), c->stream);
  if (e != cudaSuccess) return bail(LEXGB_ERR_CUDA, std::string("memset: ") + cudaGetErrorString(e));
  float* p = c->arena;
  auto take = [&]() {
    float* r = p;
    p += c->fstride;
    return r;
  };
  c->A = fields_at(take(), c->fstride);
  for (int i = 0; i < NFIELD - 1; ++i) take();
  c->B = fields_at(take(), c->fstride);
  for (int i = 0; i < NFIELD - 1; ++i) take();
  c->C = fields_at(take(), c->fstride);
  for (int i = 0; i < NFIELD - 1; ++i) take();
  c->Xu = take(); c->Xv = take(); c->Xw = take(); c->Xp = take();
  c->Yu = take(); c->Yv = take(); c->Yw = take(); c->Yp = take();
  c->Ru = take(); c->Rv = take(); c->Rw = take(); c->trho = take(); c->div = take();
  for (int i = 0; i < 5; ++i) c->sgs[i] = take();
  for (int i = 0; i < 7; ++i) c->tau[i] = take();
  for (int i = 0; i < 3; ++i) c->diag[i] = take();
  e = cudaMalloc(&c->base64, 4 * (cfg->nz + 2) * sizeof(double));
  if (e != cudaSuccess) return bail(LEXGB_ERR_ALLOC, std::string("base columns: ") + cudaGetErrorString(e));
  e = cudaMalloc(&c->tab, kColumnRows * (cfg->nz + 2) * sizeof(float));
  if (e != cudaSuccess) return bail(LEXGB_ERR_ALLOC, std::string("column table: ") + cudaGetErrorString(e));
  e = cudaMalloc(&c->partial, (size_t)budget_blocks(c->d) * kBudgetSums * sizeof(double));
  if (e != cudaSuccess) return bail(LEXGB_ERR_ALLOC, std::string("budget partials: ") + cudaGetErrorString(e));
  e = cudaMalloc(&c->budget, kBudgetSums * sizeof(double));
  if (e != cudaSuccess) return bail(LEXGB_ERR_ALLOC, std::string("budget: ") + cudaGetErrorString(e));
  e = cudaMalloc(&c->count, sizeof(unsigned long long));
  if (e != cudaSuccess) return bail(LEXGB_ERR_ALLOC, std::string("counter: ") + cudaGetErrorString(e));
  e = cudaMalloc(&c->cs_bar, sizeof(double));
  if (e != cudaSuccess) return bail(LEXGB_ERR_ALLOC, std::string("Cs gradient: ") + cudaGetErrorString(e));
  e = cudaMemsetAsync(c->cs_bar, 0, sizeof(double), c->stream);
  if (e != cudaSuccess) return bail(LEXGB_ERR_CUDA, std::string("Cs gradient: ") + cudaGetErrorString(e));
  e = cudaMalloc(&c->sync, 2 * sizeof(unsigned));
  if (e != cudaSuccess) return bail(LEXGB_ERR_ALLOC, std::string("barrier word: ") + cudaGetErrorString(e));
  e = cudaMemsetAsync(c->sync, 0, 2 * sizeof(unsigned), c->stream);
  if (e != cudaSuccess) return bail(LEXGB_ERR_CUDA, std::string("memset: ") + cudaGetErrorString(e));
  e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return bail(LEXGB_ERR_CUDA, std::string("create: ") + cudaGetErrorString(e));
  if (cfg->l2_persist == 0) setup_l2_window(c);
  if (cfg->acoustic_kernel == LEXGB_ACOUSTIC_PERSISTENT) {
    // the persistent acoustic kernel where the grid fits it; a probe launch with no sub-step (it copies
    // a scratch tile onto itself) checks that cooperative launches are available in this process
    c->persist_blocks = acoustic_persist_blocks(c->d);
    if (c->persist_blocks > 0) {
      PersistIO io{};
      for (int b = 0; b < 4; ++b) {
        io.u[b] = c->Xu;
        io.v[b] = c->Xv;
        io.w[b] = c->Xw;
      }
      io.p0 = c->Xp; io.po = c->Xp;
      io.Ru = c->Ru; io.Rv = c->Rv; io.Rw = c->Rw; io.trho = c->trho; io.ps = c->Xp;
      io.hb[0] = io.hb[1] = c->Yp;
      io.bar = c->sync;
      io.status = reinterpret_cast<int*>(c->sync + 1);
      io.spin_limit = c->spin_limit;
      io.nsub = 0;
      io.dtau = 0.f;
      e = launch_acoustic_persist(c->d, c->ph, c->cols, io, c->stream);
      if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
      if (e != cudaSuccess) {
        cudaGetLastError();
        c->persist_blocks = 0;   // one launch per sub-step instead
      }
    }
  }
  // AUTO is the rows form: measured on GB300 it is the fastest at every grid tried (192x192x96: 33.0 us
  // per sub-step against 41.8 us tiled and 49 us persistent; 32^3 to 128x128x64 likewise)
  c->ak = c->persist_blocks > 0 ? LEXGB_ACOUSTIC_PERSISTENT
          : (cfg->acoustic_kernel == LEXGB_ACOUSTIC_TILE && acoustic_tile_fits(c->d)) ? LEXGB_ACOUSTIC_TILE
                                                                                       : LEXGB_ACOUSTIC_ROWS;
  *out = c;
  return LEXGB_OK;
}

int lexgb_destroy(lexgb_ctx* c) {
  if (!c) return LEXGB_OK;
  if (c->stream) cudaStreamSynchronize(c->stream);
  drop_graph(c);
  if (c->l2on) cudaCtxResetPersistingL2Cache();  // return the persisting lines to normal use
  cudaFree(c->arena);
  cudaFree(c->sync);
  cudaFree(c->rec_arena);
  cudaFree(c->adj_arena);
  cudaFree(c->sgs_arena);
  cudaFree(c->base64);
  cudaFree(c->tab);
  cudaFree(c->stage);
  cudaFree(c->partial);
  cudaFree(c->budget);
  cudaFree(c->count);
  cudaFree(c->cs_bar);
  if (c->own_stream) cudaStreamDestroy(c->own_stream);
  if (c->copy_stream) cudaStreamDestroy(c->copy_stream);
  for (int f = 0; f < NFIELD; ++f)
    if (c->field_ev[f]) cudaEventDestroy(c->field_ev[f]);
  delete c;
  return LEXGB_OK;
}

int lexgb_set_stream(lexgb_ctx* c, void* stream) {
  if (!c) return fail(LEXGB_ERR_ARG, "null context");
  CK(cudaStreamSynchronize(c->stream));
  c->stream = stream ? (cudaStream_t)stream : c->own_stream;
  drop_graph(c);
  return LEXGB_OK;
}

int lexgb_set_base_columns(lexgb_ctx* c, const double* theta0, const double* qv0, const double* pi0,
                           const double* rho0) {
  if (!c || !theta0 || !qv0 || !pi0 || !rho0) return fail(LEXGB_ERR_ARG, "null argument");
  const size_t S = c->d.nz + 2;
  for (size_t k = 0; k < S; ++k)
    if (!(theta0[k] > 0) || !(rho0[k] > 0) || !(pi0[k] > 0) || !isfinite(qv0[k]))
      return fail(LEXGB_ERR_ARG, "base columns must be finite with positive theta0, pi0, rho0");
  const double* src[4] = {theta0, qv0, pi0, rho0};
  for (int a = 0; a < 4; ++a)
    CK(cudaMemcpyAsync(c->base64 + a * S, src[a], S * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  return build_table(c);
}

int lexgb_integrate_base_state(lexgb_ctx* c, const double* theta0, const double* qv0, double* pi0_out,
                               double* rho0_out) {
  if (!c || !theta0 || !qv0) return fail(LEXGB_ERR_ARG, "null argument");
  const size_t S = c->d.nz + 2;
  CK(cudaMemcpyAsync(c->base64, theta0, S * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  CK(cudaMemcpyAsync(c->base64 + S, qv0, S * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  CK(launch_hydrostatic(c->d.nz, c->cfg.dz, c->base64, c->base64 + S, c->base64 + 2 * S, c->base64 + 3 * S,
                        c->stream));
  CKS(build_table(c));
  if (pi0_out)
    CK(cudaMemcpyAsync(pi0_out, c->base64 + 2 * S, S * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  if (rho0_out)
    CK(cudaMemcpyAsync(rho0_out, c->base64 + 3 * S, S * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  return LEXGB_OK;
}

int lexgb_upload_state(lexgb_ctx* c, const void* const fields[6], int dtype) {
  NvtxRange nvtx_range("lexgb_upload_state");
  if (!c || !fields) return fail(LEXGB_ERR_ARG, "null argument");
  if (dtype != LEXGB_F32 && dtype != LEXGB_F64) return fail(LEXGB_ERR_ARG, "dtype must be LEXGB_F32 or LEXGB_F64");
  if (!c->base_set) return fail(LEXGB_ERR_STATE, "set the base state before uploading (theta_ref comes from it)");
  const size_t esz = dtype == LEXGB_F64 ? 8 : 4;
  size_t off[NFIELD + 1] = {0};
  for (int f = 0; f < NFIELD; ++f) {
    if (!fields[f]) return fail(LEXGB_ERR_ARG, "null field pointer");
    off[f + 1] = off[f] + (padded_count(c->d, kind_of(f)) * esz + 255) / 256 * 256;
  }
  CKS(ensure_stage(c, off[NFIELD]));
  // the copies run on the copy stream after the compute stream's earlier work (which may still
  // read the staging buffer); each field's conversion waits for its copy
  CK(cudaEventRecord(c->field_ev[0], c->stream));
  CK(cudaStreamWaitEvent(c->copy_stream, c->field_ev[0], 0));
  for (int f = 0; f < NFIELD; ++f) {
    char* dst = (char*)c->stage + off[f];
    CK(cudaMemcpyAsync(dst, fields[f], padded_count(c->d, kind_of(f)) * esz, cudaMemcpyHostToDevice,
                       c->copy_stream));
    CK(cudaEventRecord(c->field_ev[f], c->copy_stream));
  }
  for (int f = 0; f < NFIELD; ++f) {
    CK(cudaStreamWaitEvent(c->stream, c->field_ev[f], 0));
    CK(launch_import_padded(c->d, (char*)c->stage + off[f], dtype == LEXGB_F64, kind_of(f),
                            f == 0 ? c->theta_ref : 0.0, field_of(c->A, f), c->stream));
  }
  CK(cudaStreamSynchronize(c->stream));
  c->state_set = true;
  c->recorded = false;
  return LEXGB_OK;
}

int lexgb_download_state(lexgb_ctx* c, void* const fields[6], int dtype) {
  NvtxRange nvtx_range("lexgb_download_state");
  CKS(check_ready(c));
  if (!fields) return fail(LEXGB_ERR_ARG, "null argument");
  if (dtype != LEXGB_F32 && dtype != LEXGB_F64) return fail(LEXGB_ERR_ARG, "dtype must be LEXGB_F32 or LEXGB_F64");
  const size_t esz = dtype == LEXGB_F64 ? 8 : 4;
  size_t off[NFIELD + 1] = {0};
  for (int f = 0; f < NFIELD; ++f) off[f + 1] = off[f] + (padded_count(c->d, kind_of(f)) * esz + 255) / 256 * 256;
  CKS(ensure_stage(c, off[NFIELD]));
  // each field's conversion on the compute stream, its copy on the copy stream after it, so that
  // a copy overlaps the next field's conversion
  for (int f = 0; f < NFIELD; ++f) {
    if (!fields[f]) continue;
    char* src = (char*)c->stage + off[f];
    CK(launch_export_padded(c->d, field_of(c->A, f), kind_of(f), f == 0 ? c->theta_ref : 0.0, src,
                            dtype == LEXGB_F64, c->stream));
    CK(cudaEventRecord(c->field_ev[f], c->stream));
    CK(cudaStreamWaitEvent(c->copy_stream, c->field_ev[f], 0));
    CK(cudaMemcpyAsync(fields[f], src, padded_count(c->d, kind_of(f)) * esz, cudaMemcpyDeviceToHost,
                       c->copy_stream));
  }
  CK(cudaStreamSynchronize(c->copy_stream));
  CK(cudaStreamSynchronize(c->stream));
  return take_status(c);
}

int lexgb_step(lexgb_ctx* c, int nsteps, int use_graph) {
  NvtxRange nvtx_range("lexgb_step");
  CKS(check_ready(c));
  if (nsteps < 0) return fail(LEXGB_ERR_ARG, "nsteps must be >= 0");
  c->recorded = false;
  if (!use_graph) {
    for (int n = 0; n < nsteps; ++n) CKS(run_big_step(c));
    return LEXGB_OK;
  }
  if (!c->gexec) {
    // capture on the context's own stream (the legacy default stream cannot be captured); the
    // graph is then launched on whichever stream is bound
    cudaStream_t bound = c->stream;
    c->stream = c->own_stream;
    cudaError_t e = cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) {
      c->stream = bound;
      return fail(LEXGB_ERR_CUDA, std::string("graph capture: ") + cudaGetErrorString(e));
    }
    const int st = run_big_step(c);
    cudaGraph_t g = nullptr;
    e = cudaStreamEndCapture(c->stream, &g);
    c->stream = bound;
    if (st != LEXGB_OK) {
      if (g) cudaGraphDestroy(g);
      return st;
    }
    if (e != cudaSuccess) return fail(LEXGB_ERR_CUDA, std::string("graph capture: ") + cudaGetErrorString(e));
    c->graph = g;
    CK(cudaGraphInstantiate(&c->gexec, c->graph, 0));
  }
  for (int n = 0; n < nsteps; ++n) CK(cudaGraphLaunch(c->gexec, c->stream));
  return LEXGB_OK;
}

int lexgb_set_sgs_net(lexgb_ctx* c, const void* const w[4], const float* const b[4], const float* in_lo,
                      const float* in_range, const float* out_range, int enable) {
  if (!c) return fail(LEXGB_ERR_ARG, "null context");
  if (!enable) {
    if (c->sgs_on) {
      CK(cudaStreamSynchronize(c->stream));
      drop_graph(c);
    }
    c->sgs_on = false;
    return LEXGB_OK;
  }
  const Dims& d = c->d;
  if (d.nx % 16) return fail(LEXGB_ERR_ARG, "lexgb_set_sgs_net: nx must be a multiple of 16");
  if (!w || !b || !in_lo || !in_range || !out_range) return fail(LEXGB_ERR_ARG, "lexgb_set_sgs_net: null argument");
  for (int l = 0; l < 4; ++l)
    if (!w[l] || !b[l]) return fail(LEXGB_ERR_ARG, "lexgb_set_sgs_net: null weight or bias");
  const size_t cells = (size_t)d.cells();
  auto up = [](size_t n) { return (n + 255) & ~(size_t)255; };
  size_t wbytes[4], off = 0;
  size_t o_w[4], o_b[4];
  for (int l = 0; l < 4; ++l) {
    wbytes[l] = (size_t)27 * SGS_COUT[l] * SGS_CIN[l] * 2;
    o_w[l] = off;
    off += up(wbytes[l]);
    o_b[l] = off;
    off += up(SGS_COUT[l] * sizeof(float));
  }
  const size_t levels = (size_t)d.nz + 1, rcount = 5 * (size_t)d.plane() * levels;
  const size_t o_lo = off, o_rin = (off += up(5 * levels * sizeof(float))), o_rout = (off += up(5 * levels * sizeof(float)));
  const size_t o_corr = (off += up(rcount * sizeof(float)));
  const size_t o_x = (off += up(8 * cells * sizeof(float)));
  const size_t o_a0 = (off += up(cells * 16 * 2));
  const size_t o_a1 = (off += up(cells * 32 * 2));
  off += up(cells * 32 * 2);
  if (!c->sgs_arena) {
    cudaError_t e = cudaMalloc(&c->sgs_arena, off);
    if (e != cudaSuccess) {
      c->sgs_arena = nullptr;
      return fail(LEXGB_ERR_ALLOC, std::string("learned SGS buffers: ") + cudaGetErrorString(e));
    }
    char* a = c->sgs_arena;
    for (int l = 0; l < 4; ++l) {
      c->sgs_w[l] = a + o_w[l];
      c->sgs_b[l] = (float*)(a + o_b[l]);
    }
    c->sgs_lo = (float*)(a + o_lo);
    c->sgs_rin = (float*)(a + o_rin);
    c->sgs_rout = (float*)(a + o_rout);
    c->sgs_corr = (float*)(a + o_corr);
    c->sgs_x = a + o_x;
    c->sgs_a0 = a + o_a0;
    c->sgs_a1 = a + o_a1;
  }
  for (int l = 0; l < 4; ++l) {
    CK(cudaMemcpyAsync(c->sgs_w[l], w[l], wbytes[l], cudaMemcpyDeviceToDevice, c->stream));
    CK(cudaMemcpyAsync(c->sgs_b[l], b[l], SGS_COUT[l] * sizeof(float), cudaMemcpyDeviceToDevice, c->stream));
  }
  CK(cudaMemcpyAsync(c->sgs_lo, in_lo, 5 * levels * sizeof(float), cudaMemcpyDeviceToDevice, c->stream));
  CK(cudaMemcpyAsync(c->sgs_rin, in_range, 5 * levels * sizeof(float), cudaMemcpyDeviceToDevice, c->stream));
  CK(cudaMemcpyAsync(c->sgs_rout, out_range, rcount * sizeof(float), cudaMemcpyDeviceToDevice, c->stream));
  CK(conv_prepare());
  if (!c->sgs_on) {
    CK(cudaStreamSynchronize(c->stream));
    drop_graph(c);
  }
  c->sgs_on = true;
  return LEXGB_OK;
}

int lexgb_set_cs(lexgb_ctx* c, double cs) {
  if (!c) return fail(LEXGB_ERR_ARG, "null context");
  if (!(cs > 0.0)) return fail(LEXGB_ERR_ARG, "cs must be positive");
  CK(cudaStreamSynchronize(c->stream));
  const double l = cs * cbrt(c->cfg.dx * c->cfg.dy * c->cfg.dz);
  c->cs = cs;
  c->ph.smag_l2 = (float)(l * l);
  c->adj_kept = false;  // a kept step used the previous constant
  drop_graph(c);
  return LEXGB_OK;
}

int lexgb_get_cs_grad(lexgb_ctx* c, double* grad, int reset) {
  if (!c || !grad) return fail(LEXGB_ERR_ARG, "null argument");
  CK(cudaMemcpyAsync(grad, c->cs_bar, sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  if (reset) CK(cudaMemsetAsync(c->cs_bar, 0, sizeof(double), c->stream));
  CK(cudaStreamSynchronize(c->stream));
  return LEXGB_OK;
}

int lexgb_step_record(lexgb_ctx* c) {
  CKS(check_ready(c));
  CKS(ensure_record(c));
  CKS(copy_state(c, c->R0, c->A));
  if (c->cfg.turb_opt == 1) CKS(run_smag(c, c->A, nullptr, nullptr));
  CKS(run_stage(c, 0, c->A, c->A, c->S[0], c->recdT[0], c->recdq[0]));
  CKS(run_stage(c, 1, c->A, c->S[0], c->S[1], c->recdT[1], c->recdq[1]));
  CKS(run_stage(c, 2, c->A, c->S[1], c->S[2], c->recdT[2], c->recdq[2]));
  CKS(copy_state(c, c->A, c->S[2]));
  CK(cudaStreamSynchronize(c->stream));
  c->recorded = true;
  return LEXGB_OK;
}

int lexgb_download_stage(lexgb_ctx* c, int stage, double* const fields[6], double* const tends[6]) {
  CKS(check_ready(c));
  if (!c->recorded) return fail(LEXGB_ERR_STATE, "no recorded step (call lexgb_step_record first)");
  if (stage < 0 || stage > 2) return fail(LEXGB_ERR_ARG, "stage must be 0, 1 or 2");
  const StagePlan p = plan_of(c->cfg);
  size_t maxp = 0;
  for (int f = 0; f < NFIELD; ++f) maxp = padded_count(c->d, kind_of(f)) > maxp ? padded_count(c->d, kind_of(f)) : maxp;
  CKS(ensure_stage(c, 2 * maxp * sizeof(double)));
  double* s0 = (double*)c->stage;
  double* s1 = s0 + maxp;
  std::vector<double> h0, h1;
  for (int f = 0; f < NFIELD; ++f) {
    const int kd = kind_of(f);
    const double off = f == 0 ? c->theta_ref : 0.0;
    if (fields && fields[f]) {
      CK(launch_export_padded(c->d, field_of(c->S[stage], f), kd, off, s0, 1, c->stream));
      CK(cudaMemcpyAsync(fields[f], s0, padded_count(c->d, kd) * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
      CK(cudaStreamSynchronize(c->stream));
    }
    if (!tends || !tends[f]) continue;
    const size_t n = interior_count(c->d, kd);
    if (f == 0 || f == 5) {  // d_theta_dt / d_qv_dt recorded by the scalar kernel
      CK(launch_export_interior(c->d, f == 0 ? c->recdT[stage] : c->recdq[stage], kd, 0.0, s0, c->stream));
      CK(cudaMemcpyAsync(tends[f], s0, n * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
      CK(cudaStreamSynchronize(c->stream));
    } else {  // (x_stage - x0) / dt_stage, one_step_integration.py:157-160
      CK(launch_export_interior(c->d, field_of(c->S[stage], f), kd, 0.0, s0, c->stream));
      CK(launch_export_interior(c->d, field_of(c->R0, f), kd, 0.0, s1, c->stream));
      h0.resize(n);
      h1.resize(n);
      CK(cudaMemcpyAsync(h0.data(), s0, n * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
      CK(cudaMemcpyAsync(h1.data(), s1, n * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
      CK(cudaStreamSynchronize(c->stream));
      for (size_t t = 0; t < n; ++t) tends[f][t] = (h0[t] - h1[t]) / p.dts[stage];
    }
  }
  return LEXGB_OK;
}

int lexgb_diagnose(lexgb_ctx* c, int what, double* host_out) {
  CKS(check_ready(c));
  if (!host_out) return fail(LEXGB_ERR_ARG, "null output");
  if (what < 0 || what >= LEXGB_DIAG_COUNT) return fail(LEXGB_ERR_ARG, "unknown diagnostic");
  const Dims& d = c->d;
  Phys ph = c->ph;
  ph.cor_opt = 0;  // pure advection
  float* out = c->diag[0];
  int kind = 0;
  CK(launch_div_trho(d, ph, c->cols, c->A, c->div, c->trho, c->stream));
  const Sgs none{nullptr, nullptr, nullptr, nullptr, nullptr};
  switch (what) {
    case LEXGB_DIAG_MASS_DIV: out = c->div; break;
    case LEXGB_DIAG_THETA_RHO: out = c->trho; break;
    case LEXGB_DIAG_ADV_THETA:
    case LEXGB_DIAG_ADV_QV: {
      SlowOut so{nullptr, nullptr, nullptr, nullptr, nullptr, c->diag[0], c->diag[1]};
      CK(launch_adv_scalars(d, ph, c->cols, c->A, c->div, c->A.T, c->A.q, none, 0.f, so, c->stream));
      out = what == LEXGB_DIAG_ADV_THETA ? c->diag[0] : c->diag[1];
      break;
    }
    case LEXGB_DIAG_ADV_U:
    case LEXGB_DIAG_ADV_V:
    case LEXGB_DIAG_ADV_W:
    case LEXGB_DIAG_BUOY_W:
      CK(launch_adv_momentum(d, ph, c->cols, c->A, c->div, none, c->diag[0], c->diag[1], c->diag[2],
                             what == LEXGB_DIAG_BUOY_W ? 2 : 1, c->stream));
      kind = what == LEXGB_DIAG_ADV_U ? 1 : (what == LEXGB_DIAG_ADV_V ? 2 : 3);
      out = c->diag[kind - 1];
      break;
    case LEXGB_DIAG_PGF_U:
    case LEXGB_DIAG_PGF_V:
    case LEXGB_DIAG_PGF_W:
      CK(launch_diag_pgf(d, ph, c->cols, c->A.p, c->trho, c->diag[0], c->diag[1], c->diag[2], c->stream));
      kind = what - LEXGB_DIAG_PGF_U + 1;
      out = c->diag[what - LEXGB_DIAG_PGF_U];
      break;
    case LEXGB_DIAG_ADV_PI:
      CK(launch_diag_advpi(d, ph, c->cols, c->A.p, c->A.u, c->A.v, c->A.w, out, c->stream));
      break;
    case LEXGB_DIAG_SGS_U:
    case LEXGB_DIAG_SGS_V:
    case LEXGB_DIAG_SGS_W:
    case LEXGB_DIAG_SGS_THETA:
    case LEXGB_DIAG_SGS_QV:
    case LEXGB_DIAG_N2:
    case LEXGB_DIAG_KM: {
      CKS(run_smag(c, c->A, c->diag[1], c->diag[2]));
      if (what == LEXGB_DIAG_N2) {
        out = c->diag[1];
      } else if (what == LEXGB_DIAG_KM) {
        out = c->diag[2];
      } else {
        const int m = what - LEXGB_DIAG_SGS_U;
        out = c->sgs[m];
        kind = m < 3 ? m + 1 : 0;
      }
      break;
    }
    default: return fail(LEXGB_ERR_ARG, "unknown diagnostic");
  }
  const size_t n = interior_count(d, kind);
  CKS(ensure_stage(c, n * sizeof(double)));
  CK(launch_export_interior(d, out, kind, 0.0, (double*)c->stage, c->stream));
  CK(cudaMemcpyAsync(host_out, c->stage, n * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  return LEXGB_OK;
}

int lexgb_budget(lexgb_ctx* c, double* out, int n_out) {
  CKS(check_ready(c));
  if (!out || n_out < 4) return fail(LEXGB_ERR_ARG, "budget needs an output array of at least 4 doubles");
  const size_t S = c->d.nz + 2;
  CK(launch_budget(c->d, c->ph, c->cols, c->A, c->base64 + 3 * S, c->base64 + 2 * S, c->theta_ref, c->partial,
                   c->budget, c->stream));
  CK(cudaMemcpyAsync(out, c->budget, (n_out < kBudgetSums ? n_out : kBudgetSums) * sizeof(double),
                     cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  return LEXGB_OK;
}

int lexgb_check_finite(lexgb_ctx* c, long long* n_bad) {
  CKS(check_ready(c));
  if (!n_bad) return fail(LEXGB_ERR_ARG, "null output");
  CK(cudaMemsetAsync(c->count, 0, sizeof(unsigned long long), c->stream));
  for (int f = 0; f < NFIELD; ++f)
    CK(launch_count_nonfinite(field_of(c->A, f), f == 3 ? c->d.faces() : c->d.cells(), c->count, c->stream));
  unsigned long long h = 0;
  CK(cudaMemcpyAsync(&h, c->count, sizeof(h), cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  *n_bad = (long long)h;
  return take_status(c);
}

int lexgb_synchronize(lexgb_ctx* c) {
  if (!c) return fail(LEXGB_ERR_ARG, "null context");
  CK(cudaStreamSynchronize(c->stream));
  return take_status(c);
}

int lexgb_acoustic_kernel(lexgb_ctx* c, int* kind) {
  if (!c || !kind) return fail(LEXGB_ERR_ARG, "null argument");
  *kind = c->ak;
  return LEXGB_OK;
}

int lexgb_set_barrier_limit(lexgb_ctx* c, long long polls) {
  if (!c) return fail(LEXGB_ERR_ARG, "null context");
  c->barrier_test = polls < 0;
  c->spin_limit = polls == 0 ? (1LL << 24) : (polls < 0 ? -polls : polls);
  drop_graph(c);   // the limit is a kernel argument captured in the step graph
  return LEXGB_OK;
}

int lexgb_state_device_ptrs(lexgb_ctx* c, void* ptrs[6]) {
  if (!c || !ptrs) return fail(LEXGB_ERR_ARG, "null argument");
  for (int f = 0; f < NFIELD; ++f) ptrs[f] = field_of(c->A, f);
  return LEXGB_OK;
}

int lexgb_step_kernel_count(lexgb_ctx* c, int* n_kernels) {
  CKS(check_ready(c));
  if (!n_kernels) return fail(LEXGB_ERR_ARG, "null output");
  if (!c->gexec) CKS(lexgb_step(c, 0, 1));
  size_t n = 0;
  CK(cudaGraphGetNodes(c->graph, nullptr, &n));
  std::vector<cudaGraphNode_t> nodes(n);
  CK(cudaGraphGetNodes(c->graph, nodes.data(), &n));
  int k = 0;
  for (size_t i = 0; i < n; ++i) {
    cudaGraphNodeType t;
    CK(cudaGraphNodeGetType(nodes[i], &t));
    k += t == cudaGraphNodeTypeKernel;
  }
  *n_kernels = k;
  return LEXGB_OK;
}

int lexgb_time_kernel(lexgb_ctx* c, int which, int reps, float* ms_per_launch) {
  CKS(check_ready(c));
  if (!ms_per_launch || reps < 1) return fail(LEXGB_ERR_ARG, "need reps >= 1 and an output");
  if (which < 0 || which >= LEXGB_KERNEL_COUNT) return fail(LEXGB_ERR_ARG, "unknown kernel");
  const Dims& d = c->d;
  const StagePlan p = plan_of(c->cfg);
  if (which == LEXGB_KERNEL_ACOUSTIC_STAGE && (c->persist_blocks == 0 || p.n[2] < 2))
    return fail(LEXGB_ERR_STATE, "the persistent acoustic kernel is not used for this grid or configuration");
  const State& x = c->A;
  // inputs that the timed kernels read: slow tendencies of the current state
  CK(launch_div_trho(d, c->ph, c->cols, x, c->div, c->trho, c->stream));
  SmagTau t{c->tau[0], c->tau[1], c->tau[2], c->tau[3], c->tau[4], c->tau[5], c->tau[6], nullptr, nullptr};
  const Sgs sg{c->sgs[0], c->sgs[1], c->sgs[2], c->sgs[3], c->sgs[4]};
  SlowOut so{nullptr, nullptr, nullptr, c->B.T, c->B.q, nullptr, nullptr};
  const AcousticOut X{c->Xu, c->Xv, c->Xw, c->Xp}, Y{c->Yu, c->Yv, c->Yw, c->Yp};
  AcousticIn in{x.u, x.v, x.w, x.p, c->Ru, c->Rv, c->Rw, c->trho, x.p};
  auto launch = [&](int r) -> cudaError_t {
    switch (which) {
      case LEXGB_KERNEL_ACOUSTIC: {
        const AcousticOut o = (r & 1) ? Y : X;
        cudaError_t e = sub_step(c, in, o, (float)p.dtau[2], r & 1, nullptr);
        in.u = o.u; in.v = o.v; in.w = o.w; in.p = o.p;
        return e;
      }
      case LEXGB_KERNEL_ACOUSTIC_PAIR: {
        const AcousticOut o = (r & 1) ? Y : X;
        cudaError_t e = launch_acoustic_pair(d, c->ph, c->cols, in, o, (float)p.dtau[2], c->stream);
        in.u = o.u; in.v = o.v; in.w = o.w; in.p = o.p;
        return e;
      }
      case LEXGB_KERNEL_ACOUSTIC_STAGE: {   // stage 2's sub-steps from the state into scratch state C
        PersistIO io{};
        io.u[0] = x.u; io.u[1] = c->Xu; io.u[2] = c->Yu; io.u[3] = c->C.u;
        io.v[0] = x.v; io.v[1] = c->Xv; io.v[2] = c->Yv; io.v[3] = c->C.v;
        io.w[0] = x.w; io.w[1] = c->Xw; io.w[2] = c->Yw; io.w[3] = c->C.w;
        io.p0 = x.p; io.po = c->C.p;
        io.Ru = c->Ru; io.Rv = c->Rv; io.Rw = c->Rw; io.trho = c->trho; io.ps = x.p;
        io.hb[0] = c->Xp; io.hb[1] = c->Yp;
        io.bar = c->sync;
        io.status = reinterpret_cast<int*>(c->sync + 1);
        io.spin_limit = c->spin_limit;
        io.nsub = p.n[2];
        io.dtau = (float)p.dtau[2];
        return launch_acoustic_persist(d, c->ph, c->cols, io, c->stream, c->l2on ? &c->l2win : nullptr);
      }
      case LEXGB_KERNEL_DIV_TRHO: return launch_div_trho(d, c->ph, c->cols, x, c->div, c->trho, c->stream);
      case LEXGB_KERNEL_ADV_SCALARS:   // as a stage runs it: also forming div(rho0 u) and theta_rho
        return launch_adv_scalars(d, c->ph, c->cols, x, nullptr, x.T, x.q, sg, (float)p.dts[2], so, c->stream,
                                  c->div, c->trho);
      case LEXGB_KERNEL_ADV_MOMENTUM:
        return launch_adv_momentum(d, c->ph, c->cols, x, c->div, sg, c->Ru, c->Rv, c->Rw, 0, c->stream);
      case LEXGB_KERNEL_SMAG_A: return launch_smag_a(d, c->ph, c->cols, x, t, c->stream);
      default: {
        SgsOut o{c->sgs[0], c->sgs[1], c->sgs[2], c->sgs[3], c->sgs[4]};
        return launch_smag_b(d, c->ph, c->cols, x, t, o, c->stream);
      }
    }
  };
  // populate every input the timed kernel reads, then warm up once
  CK(launch_smag_a(d, c->ph, c->cols, x, t, c->stream));
  {
    const Sgs none{nullptr, nullptr, nullptr, nullptr, nullptr};
    CK(launch_adv_momentum(d, c->ph, c->cols, x, c->div, none, c->Ru, c->Rv, c->Rw, 0, c->stream));
  }
  CK(launch(0));
  in = AcousticIn{x.u, x.v, x.w, x.p, c->Ru, c->Rv, c->Rw, c->trho, x.p};
  cudaEvent_t e0, e1;
  CK(cudaEventCreate(&e0));
  CK(cudaEventCreate(&e1));
  CK(cudaEventRecord(e0, c->stream));
  for (int r = 0; r < reps; ++r) CK(launch(r));
  CK(cudaEventRecord(e1, c->stream));
  CK(cudaEventSynchronize(e1));
  float ms = 0.f;
  CK(cudaEventElapsedTime(&ms, e0, e1));
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  *ms_per_launch = ms / reps;
  return take_status(c);
}

// ------------------------------------------------------------------------------------------------
// state in the device layout (interior only, x fastest), theta in K
// ------------------------------------------------------------------------------------------------
int lexgb_set_state_interior(lexgb_ctx* c, const float* const fields[6], int on_device) {
  if (!c || !fields) return fail(LEXGB_ERR_ARG, "null argument");
  if (!c->base_set) return fail(LEXGB_ERR_STATE, "base state not set");
  for (int f = 0; f < NFIELD; ++f) {
    if (!fields[f]) return fail(LEXGB_ERR_ARG, "null field pointer");
    const size_t n = (f == 3 ? c->d.faces() : c->d.cells()) * sizeof(float);
    CK(cudaMemcpyAsync(field_of(c->A, f), fields[f], n, on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice,
                       c->stream));
  }
  if (on_device != 2) CK(launch_shift(c->A.T, -(float)c->theta_ref, (size_t)c->d.cells(), c->stream));
  c->state_set = true;
  if (!on_device) CK(cudaStreamSynchronize(c->stream));
  return LEXGB_OK;
}

int lexgb_get_state_interior(lexgb_ctx* c, float* fields[6], int on_device) {
  CKS(check_ready(c));
  if (!fields) return fail(LEXGB_ERR_ARG, "null argument");
  for (int f = 0; f < NFIELD; ++f) {
    if (!fields[f]) return fail(LEXGB_ERR_ARG, "null field pointer");
    const size_t n = (f == 3 ? c->d.faces() : c->d.cells()) * sizeof(float);
    if (f == 0 && on_device == 1) {
      CK(cudaMemcpyAsync(fields[0], c->A.T, n, cudaMemcpyDeviceToDevice, c->stream));
      CK(launch_shift(fields[0], (float)c->theta_ref, (size_t)c->d.cells(), c->stream));
      continue;
    }
    CK(cudaMemcpyAsync(fields[f], field_of(c->A, f), n, on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost,
                       c->stream));
  }
  if (!on_device) {
    CK(cudaStreamSynchronize(c->stream));
    const size_t n = (size_t)c->d.cells();
    for (size_t t = 0; t < n; ++t) fields[0][t] += (float)c->theta_ref;
    return take_status(c);
  }
  return LEXGB_OK;
}

// ------------------------------------------------------------------------------------------------
// reverse mode
// ------------------------------------------------------------------------------------------------
namespace {

struct AdjWork {
  State S[4];            // stage outputs S[1..3] (u, v, w, p alias the last acoustic state of the stage)
  float *div[3], *trho[3], *Ru[3], *Rv[3], *Rw[3];
  float* ac[3][64][4];   // acoustic states 1..n of each stage: u, v, w, p
  State Xb0, Cur, Xs;    // adjoints: step input, current stage output, current stage input
  State X0;              // input state of a kept step (lexgb_step_keep)
  float* pp[2][4];       // acoustic adjoint ping-pong
  float *Rub, *Rvb, *Rwb, *trhob, *psb;
  float* cb[5];
  float* divb;
  float* P[5][6];
  float* mb[4];
  float* sgsb[5];
  SmagLin sl;
  SmagVjpArgs sv;
};

int adj_fields(const StagePlan& p) { return 6 + 15 + 4 * (p.n[0] + p.n[1] + p.n[2]) + 18 + 8 + 5 + 6 + 34 + 5 + 22 + 6 + 1; }

int ensure_adjoint(lexgb_ctx* c, AdjWork& w) {
  const StagePlan p = plan_of(c->cfg);
  if (p.n[0] > 64 || p.n[1] > 64 || p.n[2] > 64) return fail(LEXGB_ERR_ARG, "adjoint supports up to 64 acoustic sub-steps per stage");
  const size_t nf = adj_fields(p);
  if (!c->adj_arena) {
    cudaError_t e = cudaMalloc(&c->adj_arena, nf * c->fstride * sizeof(float));
    if (e != cudaSuccess) return fail(LEXGB_ERR_ALLOC, std::string("adjoint workspace: ") + cudaGetErrorString(e));
  }
  float* q = c->adj_arena;
  auto take = [&]() {
    float* r = q;
    q += c->fstride;
    return r;
  };
  for (int s = 0; s < 3; ++s) {
    w.div[s] = take(); w.trho[s] = take(); w.Ru[s] = take(); w.Rv[s] = take(); w.Rw[s] = take();
    for (int m = 1; m <= p.n[s]; ++m)
      for (int f = 0; f < 4; ++f) w.ac[s][m][f] = take();
    State& o = w.S[s + 1];
    o.T = take();
    o.q = take();
    o.u = w.ac[s][p.n[s]][0]; o.v = w.ac[s][p.n[s]][1]; o.w = w.ac[s][p.n[s]][2]; o.p = w.ac[s][p.n[s]][3];
  }
  w.Xb0 = fields_at(take(), c->fstride); for (int i = 1; i < NFIELD; ++i) take();
  w.Cur = fields_at(take(), c->fstride); for (int i = 1; i < NFIELD; ++i) take();
  w.Xs = fields_at(take(), c->fstride); for (int i = 1; i < NFIELD; ++i) take();
  w.X0 = fields_at(take(), c->fstride); for (int i = 1; i < NFIELD; ++i) take();
  for (int a = 0; a < 2; ++a) for (int f = 0; f < 4; ++f) w.pp[a][f] = take();
  w.Rub = take(); w.Rvb = take(); w.Rwb = take(); w.trhob = take(); w.psb = take();
  for (int f = 0; f < 5; ++f) w.cb[f] = take();
  w.divb = take();
  for (int f = 0; f < 5; ++f) for (int s = 0; s < 6; ++s) w.P[f][s] = take();
  for (int f = 0; f < 4; ++f) w.mb[f] = take();
  for (int f = 0; f < 5; ++f) w.sgsb[f] = take();
  for (int f = 0; f < 6; ++f) w.sl.s[f] = take();
  w.sl.km = take();
  w.sl.kS = take();
  for (int f = 0; f < 6; ++f) w.sv.tb[f] = take();
  w.sv.khb = take();
  for (int f = 0; f < 6; ++f) w.sv.sb[f] = take();
  w.sv.n2b = take();
  w.sv.kmkb = take();
  w.sv.gu = w.sgsb[0]; w.sv.gv = w.sgsb[1]; w.sv.gw = w.sgsb[2]; w.sv.gT = w.sgsb[3]; w.sv.gq = w.sgsb[4];
  if ((size_t)(q - c->adj_arena) > nf * c->fstride) return fail(LEXGB_ERR_STATE, "adjoint workspace layout");
  return LEXGB_OK;
}

// A persisting L2 window over [base, base + bytes) when the context uses them (l2_persist):
// the process's set-aside is raised to cover it, up to the device maximum.
bool l2_window_for(lexgb_ctx* c, void* base, size_t bytes, cudaAccessPolicyWindow* win) {
  if (!c->l2on) return false;
  int dev = 0, max_persist = 0, max_window = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&max_persist, cudaDevAttrMaxPersistingL2CacheSize, dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&max_window, cudaDevAttrMaxAccessPolicyWindowSize, dev) != cudaSuccess ||
      max_persist <= 0 || max_window <= 0) {
    cudaGetLastError();
    return false;
  }
  if (bytes > (size_t)max_window) bytes = (size_t)max_window;
  size_t want = bytes < (size_t)max_persist ? bytes : (size_t)max_persist, cur = 0;
  if (cudaDeviceGetLimit(&cur, cudaLimitPersistingL2CacheSize) != cudaSuccess) cur = 0;
  if (cur < want) {
    if (cudaDeviceSetLimit(cudaLimitPersistingL2CacheSize, want) != cudaSuccess) {
      cudaGetLastError();
      return false;
    }
    cur = want;
  }
  win->base_ptr = base;
  win->num_bytes = bytes;
  win->hitRatio = cur >= bytes ? 1.0f : (float)cur / (float)bytes;
  win->hitProp = cudaAccessPropertyPersisting;
  win->missProp = cudaAccessPropertyStreaming;
  return true;
}

int zero_state(lexgb_ctx* c, const State& s) {
  for (int f = 0; f < NFIELD; ++f) CK(cudaMemsetAsync(field_of(s, f), 0, c->fstride * sizeof(float), c->stream));
  return LEXGB_OK;
}

}  // namespace

namespace {

// forward of the first nstages stages from x0, keeping every intermediate the reverse pass reads
int adj_forward(lexgb_ctx* c, AdjWork& w, const State& x0, int nstages) {
  const Dims& d = c->d;
  const StagePlan p = plan_of(c->cfg);
  const State& A = x0;
  Sgs sg{nullptr, nullptr, nullptr, nullptr, nullptr};
  if (c->cfg.turb_opt == 1) {
    CKS(run_smag(c, A, nullptr, nullptr));
    sg = Sgs{c->sgs[0], c->sgs[1], c->sgs[2], c->sgs[3], c->sgs[4]};
  }
  for (int s = 0; s < nstages; ++s) {
    const State xs = s == 0 ? A : w.S[s];
    const State& out = w.S[s + 1];
    SlowOut so{nullptr, nullptr, nullptr, out.T, out.q, nullptr, nullptr};
    CK(launch_adv_scalars(d, c->ph, c->cols, xs, nullptr, A.T, A.q, sg, (float)p.dts[s], so, c->stream, w.div[s],
                          w.trho[s]));
    CK(launch_adv_momentum(d, c->ph, c->cols, xs, w.div[s], sg, w.Ru[s], w.Rv[s], w.Rw[s], 0, c->stream));
    AcousticIn in{A.u, A.v, A.w, A.p, w.Ru[s], w.Rv[s], w.Rw[s], w.trho[s], xs.p};
    // the stage's theta_rho, R_u, R_v, R_w (adjacent workspace fields) persist in L2 through its sub-steps
    cudaAccessPolicyWindow win{};
    const bool win_on = l2_window_for(c, w.trho[s], 4 * c->fstride * sizeof(float), &win);
    for (int m = 1; m <= p.n[s]; ++m) {
      const AcousticOut o{w.ac[s][m][0], w.ac[s][m][1], w.ac[s][m][2], w.ac[s][m][3]};
      CK(sub_step(c, in, o, (float)p.dtau[s], 0, win_on ? &win : nullptr));
      in.u = o.u; in.v = o.v; in.w = o.w; in.p = o.p;
    }
  }
  return LEXGB_OK;
}

// reverse pass over the intermediates adj_forward kept for x0
int adj_reverse(lexgb_ctx* c, AdjWork& w, const State& x0, int nstages, const float* const ybar[6], float* xbar[6],
                int on_device) {
  const Dims& d = c->d;
  const StagePlan p = plan_of(c->cfg);
  const State& A = x0;
  const bool turb = c->cfg.turb_opt == 1;
  // ---- seed
  const size_t cells = (size_t)d.cells(), faces = (size_t)d.faces();
  for (int f = 0; f < 6; ++f) {
    const size_t n = (f == 3 ? faces : cells) * sizeof(float);
    CK(cudaMemsetAsync(field_of(w.Cur, f), 0, c->fstride * sizeof(float), c->stream));
    CK(cudaMemcpyAsync(field_of(w.Cur, f), ybar[f], n, on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice,
                       c->stream));
  }
  CKS(zero_state(c, w.Xb0));
  if (turb)
    for (int f = 0; f < 5; ++f) CK(cudaMemsetAsync(w.sgsb[f], 0, c->fstride * sizeof(float), c->stream));
  // ---- reverse.  The acoustic adjoints read and write the five accumulators (adjacent fields)
  // in every sub-step: a persisting L2 window keeps them on chip through a stage.
  cudaAccessPolicyWindow awin{};
  const bool awin_on = l2_window_for(c, w.Rub, 5 * c->fstride * sizeof(float), &awin);
  for (int s = nstages - 1; s >= 0; --s) {
    const State xs = s == 0 ? A : w.S[s];
    CKS(zero_state(c, w.Xs));
    for (float* z : {w.Rub, w.Rvb, w.Rwb, w.trhob, w.psb})
      CK(cudaMemsetAsync(z, 0, c->fstride * sizeof(float), c->stream));
    // acoustic loop backwards
    const float* adj[4] = {w.Cur.u, w.Cur.v, w.Cur.w, w.Cur.p};
    for (int m = p.n[s], k = 0; m >= 1; --m, ++k) {
      float* const* o = w.pp[k & 1];
      const float* oldp = m == 1 ? A.p : w.ac[s][m - 1][3];
      AcousticVjpArgs a{oldp, w.trho[s], xs.p, w.ac[s][m][0], w.ac[s][m][1], w.ac[s][m][2],
                        adj[0], adj[1], adj[2], adj[3], o[0], o[1], o[2], o[3],
                        w.Rub, w.Rvb, w.Rwb, w.trhob, w.psb};
      CK(launch_acoustic_vjp(d, c->ph, c->cols, a, (float)p.dtau[s], c->stream, awin_on ? &awin : nullptr));
      for (int f = 0; f < 4; ++f) adj[f] = o[f];
    }
    // slow tendencies, theta/qv update, theta_rho, pi'_s; the acoustic loop's input adjoints go to
    // the big step's input adjoint in the same pass
    StageVjpArgs sa{};
    for (int f = 0; f < 4; ++f) sa.acb[f] = adj[f];
    sa.xs = xs;
    sa.div = w.div[s];
    sa.Tnb = w.Cur.T;
    sa.qnb = w.Cur.q;
    sa.Rub = w.Rub; sa.Rvb = w.Rvb; sa.Rwb = w.Rwb; sa.trhob = w.trhob; sa.psb = w.psb;
    sa.dts = (float)p.dts[s];
    sa.xsb = w.Xs;
    sa.x0b = w.Xb0;
    for (int f = 0; f < 5; ++f) sa.cb[f] = w.cb[f];
    sa.divb = w.divb;
    if (turb) {
      sa.sgsb_u = w.sgsb[0]; sa.sgsb_v = w.sgsb[1]; sa.sgsb_w = w.sgsb[2]; sa.sgsb_T = w.sgsb[3]; sa.sgsb_q = w.sgsb[4];
    }
    CK(launch_stage_pointwise_vjp(d, c->ph, c->cols, sa, c->stream));
    AdvVjpArgs aa{};
    aa.xs = xs;
    aa.phi[0] = xs.u; aa.phi[1] = xs.v; aa.phi[2] = xs.w; aa.phi[3] = xs.T; aa.phi[4] = xs.q;
    for (int f = 0; f < 5; ++f) {
      aa.cb[f] = w.cb[f];
      for (int q = 0; q < 6; ++q) aa.P[f][q] = w.P[f][q];
    }
    for (int f = 0; f < 4; ++f) aa.mb[f] = w.mb[f];
    aa.xsb = w.Xs;
    CK(launch_adv_vjp(d, c->ph, c->cols, aa, c->stream));
    // the first stage's input is the big step's input: its adjoint goes to Xb0 in the same pass
    CK(launch_massdiv_vjp(d, c->ph, c->cols, w.divb, w.Xs, c->stream, s == 0 ? w.Xb0 : State{}));
    if (s > 0) std::swap(w.Cur, w.Xs);
  }
  // the SGS tendencies were taken from the step's input state
  if (turb) {
    w.sv.x0b = w.Xb0;
    CK(launch_smag_vjp(d, c->ph, c->cols, A, w.sl, w.sv, c->stream));
    // dK_m/dCs = 2 K_m / Cs: the Cs derivative of this step
    CK(launch_sum_scaled(d.cells(), w.sv.kmkb, 2.0 / c->cs, c->cs_bar, c->stream));
  }
  for (int f = 0; f < 6; ++f) {
    const size_t n = (f == 3 ? faces : cells) * sizeof(float);
    CK(cudaMemcpyAsync(xbar[f], field_of(w.Xb0, f), n, on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost,
                       c->stream));
  }
  CK(cudaStreamSynchronize(c->stream));
  // the accumulators' persisting lines (71 MB at 192 x 192 x 96) would crowd the L2 of the work
  // that follows; return them to normal use (the step's own window re-persists its fields)
  if (awin_on) cudaCtxResetPersistingL2Cache();
  return LEXGB_OK;
}

int check_vjp_args(const float* const ybar[6], float* xbar[6]) {
  if (!ybar || !xbar) return fail(LEXGB_ERR_ARG, "need ybar and xbar");
  for (int f = 0; f < 6; ++f)
    if (!ybar[f] || !xbar[f]) return fail(LEXGB_ERR_ARG, "null field pointer");
  return LEXGB_OK;
}

}  // namespace

int lexgb_step_vjp(lexgb_ctx* c, int nstages, const float* const ybar[6], float* xbar[6], int on_device) {
  NvtxRange nvtx_range("lexgb_step_vjp");
  CKS(check_ready(c));
  if (nstages < 1 || nstages > 3) return fail(LEXGB_ERR_ARG, "need 1..3 stages");
  CKS(check_vjp_args(ybar, xbar));
  AdjWork w;
  CKS(ensure_adjoint(c, w));
  c->adj_kept = false;  // the workspace is reused below
  CKS(adj_forward(c, w, c->A, nstages));
  return adj_reverse(c, w, c->A, nstages, ybar, xbar, on_device);
}

int lexgb_step_keep(lexgb_ctx* c) {
  NvtxRange nvtx_range("lexgb_step_keep");
  CKS(check_ready(c));
  AdjWork w;
  CKS(ensure_adjoint(c, w));
  for (int f = 0; f < NFIELD; ++f)
    CK(cudaMemcpyAsync(field_of(w.X0, f), field_of(c->A, f), c->fstride * sizeof(float), cudaMemcpyDeviceToDevice,
                       c->stream));
  CKS(adj_forward(c, w, w.X0, 3));
  for (int f = 0; f < NFIELD; ++f)
    CK(cudaMemcpyAsync(field_of(c->A, f), field_of(w.S[3], f), c->fstride * sizeof(float), cudaMemcpyDeviceToDevice,
                       c->stream));
  c->adj_kept = true;
  return LEXGB_OK;
}

int lexgb_step_vjp_kept(lexgb_ctx* c, const float* const ybar[6], float* xbar[6], int on_device) {
  NvtxRange nvtx_range("lexgb_step_vjp_kept");
  CKS(check_ready(c));
  CKS(check_vjp_args(ybar, xbar));
  if (!c->adj_kept) return fail(LEXGB_ERR_STATE, "no kept step: call lexgb_step_keep first");
  AdjWork w;
  CKS(ensure_adjoint(c, w));
  return adj_reverse(c, w, w.X0, 3, ybar, xbar, on_device);
}

int lexgb_last_error(char* buf, size_t len) {
  if (buf && len) {
    const size_t n = g_last_error.size() < len - 1 ? g_last_error.size() : len - 1;
    memcpy(buf, g_last_error.data(), n);
    buf[n] = '\0';
  }
  return (int)g_last_error.size();
}

}  // extern "C"
