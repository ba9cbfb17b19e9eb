// kernels_acoustic_tile.cu - one acoustic sub-step on 32 x 4 x 8 blocks of cells
// (sound_rk_step0/1/2, one_step_integration.py:519-556, :638-675, :757-794).
//
// The same sub-step as k_acoustic_vec (u, v, w <- PGF + slow tendencies, w = 0 on the bottom and
// lid faces, pi' <- divergence + advection_pi), with each input value read from memory once per
// block instead of once per use: a thread owns 4 consecutive x points of one row and level; a warp
// is 8 such quads x 4 rows of one level, so x and y neighbours come by warp shuffles (the warp's
// edge lanes load the values beyond it), and the block's 8 warps are 8 consecutive levels, which
// exchange pi', theta_rho, pi'_s and the new bottom-face w through 16 KB of shared memory.  The
// new w on a cell's top face is the new w on the bottom face of the cell above, taken from shared
// memory (the top warp of a block computes it).  Every face and cell is evaluated with the same
// expression as in k_acoustic_vec, so the two kernels give identical results.
#include "lexgb_internal.cuh"

namespace lexgb {

namespace {

constexpr int TQ = 8, TR = 4, TL = 8, TT = TQ * TR * TL;  // 8 quads (32 columns) x 4 rows x 8 levels
constexpr unsigned FULL = 0xffffffffu;
constexpr float kHalfCpT = (float)(0.5 * kCp);
constexpr float kRdCvT = (float)(kRd / kCv);

__device__ __forceinline__ float pgft(float tra, float trb, float pa, float pb, float rd) {
  return -kHalfCpT * (tra + trb) * ((pa - pb) * rd);
}
__device__ __forceinline__ float4 ldg4(const float* p) { return __ldg(reinterpret_cast<const float4*>(p)); }
__device__ __forceinline__ void st4(float* p, float4 v) { *reinterpret_cast<float4*>(p) = v; }
__device__ __forceinline__ float4 zero4() { return make_float4(0.f, 0.f, 0.f, 0.f); }
__device__ __forceinline__ float el(const float4& v, int l) { return l == 0 ? v.x : (l == 1 ? v.y : (l == 2 ? v.z : v.w)); }
__device__ __forceinline__ float4 shup4(float4 v, int dl) {
  return make_float4(__shfl_up_sync(FULL, v.x, dl), __shfl_up_sync(FULL, v.y, dl), __shfl_up_sync(FULL, v.z, dl),
                     __shfl_up_sync(FULL, v.w, dl));
}
__device__ __forceinline__ float4 shdn4(float4 v, int dl) {
  return make_float4(__shfl_down_sync(FULL, v.x, dl), __shfl_down_sync(FULL, v.y, dl),
                     __shfl_down_sync(FULL, v.z, dl), __shfl_down_sync(FULL, v.w, dl));
}

__global__ void __launch_bounds__(TT, 2) k_acoustic_tile(Dims d, Phys ph, Cols c, AcousticIn a, AcousticOut o,
                                                         float dtau, int rev) {
  __shared__ float4 xP[TL][TR * TQ], xT[TL][TR * TQ], xS[TL][TR * TQ], xW[TL][TR * TQ];
  const int nx = d.nx, ny = d.ny, nz = d.nz, plane = nx * ny;
  const int bx = rev ? gridDim.x - 1 - blockIdx.x : blockIdx.x;
  const int by = rev ? gridDim.y - 1 - blockIdx.y : blockIdx.y;
  const int bz = rev ? gridDim.z - 1 - blockIdx.z : blockIdx.z;
  const int tid = threadIdx.x, lane = tid & 31, qx = tid & 7, jj = (tid >> 3) & 3, kk = tid >> 5;
  const int i0 = bx * 32 + 4 * qx, j = by * TR + jj, k = bz * TL + kk;
  const bool live = k < nz;   // warp-uniform
  const int kc = live ? k : nz - 1;
  const int r0 = kc * plane + j * nx + i0;
  const int jm = wrap(j - 1, ny), jp = wrap(j + 1, ny);
  const int iw = wrap(i0 - 1, nx), ie = wrap(i0 + 4, nx);
  const float rdx = ph.rdx, rdy = ph.rdy, rdz = ph.rdz;

  // ---- every load, issued before any use
  const float4 P = ldg4(a.p + r0), TRo = ldg4(a.trho + r0), S0 = ldg4(a.ps + r0);
  const float4 U = ldg4(a.u + r0), RU = ldg4(a.Ru + r0), Vv = ldg4(a.v + r0), RV = ldg4(a.Rv + r0);
  const float4 W = ldg4(a.w + r0), RW = ldg4(a.Rw + r0);
  float pWg = 0.f, tWg = 0.f, sWg = 0.f, pEg = 0.f, tEg = 0.f, uEg = 0.f, ruEg = 0.f, sEg = 0.f;
  if (qx == 0) {
    const int rw = kc * plane + j * nx + iw;
    pWg = __ldg(a.p + rw); tWg = __ldg(a.trho + rw); sWg = __ldg(a.ps + rw);
  }
  if (qx == TQ - 1) {
    const int re = kc * plane + j * nx + ie;
    pEg = __ldg(a.p + re); tEg = __ldg(a.trho + re); uEg = __ldg(a.u + re); ruEg = __ldg(a.Ru + re);
    sEg = __ldg(a.ps + re);
  }
  float4 PSg = zero4(), TSg = zero4(), SSg = zero4();
  float4 PNg = zero4(), TNg = zero4(), SNg = zero4(), VNg = zero4(), RVNg = zero4();
  if (jj == 0) {
    const int rs = kc * plane + jm * nx + i0;
    PSg = ldg4(a.p + rs); TSg = ldg4(a.trho + rs); SSg = ldg4(a.ps + rs);
  }
  if (jj == TR - 1) {
    const int rn = kc * plane + jp * nx + i0;
    PNg = ldg4(a.p + rn); TNg = ldg4(a.trho + rn); SNg = ldg4(a.ps + rn); VNg = ldg4(a.v + rn);
    RVNg = ldg4(a.Rv + rn);
  }
  const bool has_b = live && k > 0, has_t = live && k + 1 < nz;
  float4 PBg = zero4(), TBg = zero4(), SBg = zero4();
  float4 PTg = zero4(), TTg = zero4(), STg = zero4(), WTg = zero4(), RWTg = zero4();
  if (kk == 0 && has_b) {
    PBg = ldg4(a.p + r0 - plane); TBg = ldg4(a.trho + r0 - plane); SBg = ldg4(a.ps + r0 - plane);
  }
  if (kk == TL - 1 && has_t) {
    PTg = ldg4(a.p + r0 + plane); TTg = ldg4(a.trho + r0 + plane); STg = ldg4(a.ps + r0 + plane);
    WTg = ldg4(a.w + r0 + plane); RWTg = ldg4(a.Rw + r0 + plane);
  }

  // ---- levels: exchange pi', theta_rho and pi'_s with the warps above and below
  const int me = jj * TQ + qx;
  xP[kk][me] = P;
  xT[kk][me] = TRo;
  xS[kk][me] = S0;
  // x neighbours within the row of 8 quads, y neighbours within the warp's 4 rows
  float pW = __shfl_up_sync(FULL, P.w, 1, 8), tW = __shfl_up_sync(FULL, TRo.w, 1, 8);
  float sW = __shfl_up_sync(FULL, S0.w, 1, 8);
  float pE = __shfl_down_sync(FULL, P.x, 1, 8), tE = __shfl_down_sync(FULL, TRo.x, 1, 8);
  float uE = __shfl_down_sync(FULL, U.x, 1, 8), ruE = __shfl_down_sync(FULL, RU.x, 1, 8);
  float sE = __shfl_down_sync(FULL, S0.x, 1, 8);
  if (qx == 0) { pW = pWg; tW = tWg; sW = sWg; }
  if (qx == TQ - 1) { pE = pEg; tE = tEg; uE = uEg; ruE = ruEg; sE = sEg; }
  float4 PS = shup4(P, 8), TS = shup4(TRo, 8), SS = shup4(S0, 8);
  float4 PN = shdn4(P, 8), TN = shdn4(TRo, 8), SN = shdn4(S0, 8), VN = shdn4(Vv, 8), RVN = shdn4(RV, 8);
  if (jj == 0) { PS = PSg; TS = TSg; SS = SSg; }
  if (jj == TR - 1) { PN = PNg; TN = TNg; SN = SNg; VN = VNg; RVN = RVNg; }
  (void)lane;
  __syncthreads();
  const float4 PB = kk > 0 ? xP[kk - 1][me] : PBg, TB = kk > 0 ? xT[kk - 1][me] : TBg;
  const float4 SB = kk > 0 ? xS[kk - 1][me] : SBg;
  const float4 ST = kk < TL - 1 ? xS[kk + 1][me] : STg;

  // ---- new winds: u on the 4 west faces and the east face, v on the south and north faces,
  // w on the bottom face (shared with the warp below as its top face)
  float un[5];
  un[0] = U.x + (pgft(TRo.x, tW, P.x, pW, rdx) + RU.x) * dtau;
  un[1] = U.y + (pgft(TRo.y, TRo.x, P.y, P.x, rdx) + RU.y) * dtau;
  un[2] = U.z + (pgft(TRo.z, TRo.y, P.z, P.y, rdx) + RU.z) * dtau;
  un[3] = U.w + (pgft(TRo.w, TRo.z, P.w, P.z, rdx) + RU.w) * dtau;
  un[4] = uE + (pgft(tE, TRo.w, pE, P.w, rdx) + ruE) * dtau;
  float vs[4], vn[4], wb[4];
#pragma unroll
  for (int l = 0; l < 4; ++l) {
    const float p0 = el(P, l), t0 = el(TRo, l);
    vs[l] = el(Vv, l) + (pgft(t0, el(TS, l), p0, el(PS, l), rdy) + el(RV, l)) * dtau;
    vn[l] = el(VN, l) + (pgft(el(TN, l), t0, el(PN, l), p0, rdy) + el(RVN, l)) * dtau;
    wb[l] = has_b ? el(W, l) + (pgft(t0, el(TB, l), p0, el(PB, l), rdz) + el(RW, l)) * dtau : 0.f;
  }
  xW[kk][me] = make_float4(wb[0], wb[1], wb[2], wb[3]);
  __syncthreads();
  float wt[4];
  if (kk < TL - 1) {
    const float4 t = xW[kk + 1][me];
    wt[0] = t.x; wt[1] = t.y; wt[2] = t.z; wt[3] = t.w;
  } else {
#pragma unroll
    for (int l = 0; l < 4; ++l)
      wt[l] = has_t ? el(WTg, l) + (pgft(el(TTg, l), el(TRo, l), el(PTg, l), el(P, l), rdz) + el(RWTg, l)) * dtau : 0.f;
  }
  if (!live) return;
#pragma unroll
  for (int l = 0; l < 4; ++l)
    if (!has_t) wt[l] = 0.f;

  // ---- new pi' (divergence and advection_pi of the new winds)
  const float rho = c.rho[k], rhoi = c.rho_inv[k], rfb = c.rho_face[k], rft = c.rho_face[k + 1];
  const float dzb = c.dpi0dz[k], dzt = c.dpi0dz[k + 1], pi0 = c.pi0[k];
  const float sc[6] = {sW, S0.x, S0.y, S0.z, S0.w, sE};
  float outp[4];
#pragma unroll
  for (int l = 0; l < 4; ++l) {
    const float div = (un[l + 1] - un[l]) * rdx + (vn[l] - vs[l]) * rdy + (wt[l] - wb[l]) * rdz;
    const float s0 = sc[l + 1];
    const float gxw = (s0 - sc[l]) * rdx, gxe = (sc[l + 2] - s0) * rdx;
    const float gys = (s0 - el(SS, l)) * rdy, gyn = (el(SN, l) - s0) * rdy;
    const float wzb = has_b ? wb[l] * (dzb + (s0 - el(SB, l)) * rdz) : 0.f;
    const float wzt = has_t ? wt[l] * (dzt + (el(ST, l) - s0) * rdz) : 0.f;
    const float ap = -(0.5f * (un[l + 1] * gxe + un[l] * gxw) + 0.5f * (vn[l] * gyn + vs[l] * gys) +
                       (0.5f * wzb * rfb + 0.5f * wzt * rft) * rhoi);
    const float dpdt = -kRdCvT * ((pi0 + s0) * div) + ap;
    outp[l] = el(P, l) + (kDivDamp * dpdt) * dtau;
  }
  st4(o.p + r0, make_float4(outp[0], outp[1], outp[2], outp[3]));
  st4(o.u + r0, make_float4(un[0], un[1], un[2], un[3]));
  st4(o.v + r0, make_float4(vs[0], vs[1], vs[2], vs[3]));
  st4(o.w + r0, make_float4(wb[0], wb[1], wb[2], wb[3]));
  if (k == nz - 1) st4(o.w + r0 + plane, zero4());
}

}  // namespace

bool acoustic_tile_fits(const Dims& d) { return d.nx % 32 == 0 && d.ny % TR == 0; }

cudaError_t launch_acoustic_tile(const Dims& d, const Phys& ph, const Cols& c, AcousticIn in, AcousticOut out,
                                 float dtau, cudaStream_t st, int rev, const cudaAccessPolicyWindow* win) {
  const dim3 g(d.nx / 32, d.ny / TR, (d.nz + TL - 1) / TL), b(TT);
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
    return cudaLaunchKernelEx(&cfg, k_acoustic_tile, d, ph, c, in, out, dtau, rev);
  }
  k_acoustic_tile<<<g, b, 0, st>>>(d, ph, c, in, out, dtau, rev);
  return cudaGetLastError();
}

}  // namespace lexgb
