// kernels_misc.cu - layout conversion, FP64 base state, FP64 budgets, non-finite count.
#include "lexgb_internal.cuh"

namespace lexgb {

namespace {

constexpr int NGX = 3, NGY = 3, NGZ = 1;

// padded reference extents of a field kind (0 scalar, 1 u, 2 v, 3 w)
__host__ __device__ inline void padded_extents(const Dims& d, int kind, int& PX, int& PY, int& PZ) {
  PX = d.nx + 2 * NGX + (kind == 1 ? 1 : 0);
  PY = d.ny + 2 * NGY + (kind == 2 ? 1 : 0);
  PZ = d.nz + 2 * NGZ + (kind == 3 ? 1 : 0);
}

__host__ __device__ inline int levels(const Dims& d, int kind) { return kind == 3 ? d.nz + 1 : d.nz; }

// Device layout <- reference padded layout (interior part; u/v drop the duplicated face), and
// reference padded layout <- device layout with the ghosts filled as padding3_array /
// padding3u_array / padding3v_array (one_step_integration.py:950-985).  Tiled transposes: at one y
// row, a 32 x 32 tile of (x, level) goes through shared memory, so both the padded layout (level
// fastest) and the device layout (x fastest) are read and written in whole rows.  Block (32, 8),
// grid (x tiles, level tiles, rows).
constexpr int TT = 32, TR = 8;

template <typename Src>
__global__ void __launch_bounds__(TT* TR) k_import_t(Dims d, const Src* __restrict__ src, int kind, double offset,
                                                    float* __restrict__ dst) {
  __shared__ float tile[TT][TT + 1];
  int PX, PY, PZ;
  padded_extents(d, kind, PX, PY, PZ);
  const int nl = levels(d, kind), j = blockIdx.z;
  const int i0 = blockIdx.x * TT, k0 = blockIdx.y * TT, tx = threadIdx.x, ty = threadIdx.y;
  for (int r = ty; r < TT; r += TR) {   // rows x = i0 + r, levels k0 + tx along the row
    const int i = i0 + r, k = k0 + tx;
    if (i < d.nx && k < nl)
      tile[r][tx] = (float)((double)src[((long long)(i + NGX) * PY + (j + NGY)) * PZ + (k + NGZ)] - offset);
  }
  __syncthreads();
  for (int r = ty; r < TT; r += TR) {   // rows k = k0 + r, x = i0 + tx along the row
    const int i = i0 + tx, k = k0 + r;
    if (i < d.nx && k < nl) dst[(long long)k * d.plane() + (long long)j * d.nx + i] = tile[tx][r];
  }
}

template <typename Dst>
__global__ void __launch_bounds__(TT* TR) k_export_t(Dims d, const float* __restrict__ src, int kind, double offset,
                                                    Dst* __restrict__ dst) {
  __shared__ float tile[TT][TT + 1];
  int PX, PY, PZ;
  padded_extents(d, kind, PX, PY, PZ);
  const int nl = levels(d, kind), q = blockIdx.z, j = wrap(q - NGY, d.ny);
  const int p0 = blockIdx.x * TT, L0 = blockIdx.y * TT, tx = threadIdx.x, ty = threadIdx.y;
  for (int r = ty; r < TT; r += TR) {   // padded levels L0 + r, padded x p0 + tx along the row
    const int p = p0 + tx, L = L0 + r;
    if (p < PX && L < PZ)
      tile[r][tx] = src[(long long)clampi(L - NGZ, 0, nl - 1) * d.plane() + (long long)j * d.nx + wrap(p - NGX, d.nx)];
  }
  __syncthreads();
  for (int r = ty; r < TT; r += TR) {   // padded x p0 + r, levels L0 + tx along the row
    const int p = p0 + r, L = L0 + tx;
    if (p < PX && L < PZ) dst[((long long)p * PY + q) * PZ + L] = (Dst)((double)tile[tx][r] + offset);
  }
}

// interior arrays in reference C order; u (nx+1), v (ny+1), w (nz+1) staggered extents
__global__ void k_export_interior(Dims d, const float* __restrict__ src, int kind, double offset,
                                  double* __restrict__ dst) {
  const int EX = d.nx + (kind == 1 ? 1 : 0), EY = d.ny + (kind == 2 ? 1 : 0), EZ = levels(d, kind);
  const long long n = (long long)EX * EY * EZ;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
    const int k = (int)(t % EZ);
    const int j = (int)((t / EZ) % EY);
    const int i = (int)(t / ((long long)EZ * EY));
    dst[t] = (double)src[d.at(wrap(i, d.nx), wrap(j, d.ny), k)] + offset;
  }
}

// FP64 hydrostatic base state on the padded column (setup_lex.py:123-132): pi at the faces by
// cumulative sum of -g/(Cp theta_rho0) dz from pi = 1 at z = 0, cell values the face average,
// ghost levels copied from the edge levels, rho0 = pi0^(Cv/Rd) p00 / Rd / theta_rho0.
__global__ void k_hydrostatic(int nz, double dz, const double* __restrict__ th0, const double* __restrict__ q0,
                              double* __restrict__ pi0, double* __restrict__ rho0) {
  if (blockIdx.x != 0 || threadIdx.x != 0) return;
  double face_lo = 1.0, acc = 0.0;
  for (int k = 1; k <= nz; ++k) {
    const double trho0 = th0[k] * (1.0 + kReps * q0[k]) / (1.0 + q0[k]);
    acc += -kG / kCp / trho0;
    const double face_hi = acc * dz + 1.0;
    pi0[k] = 0.5 * (face_lo + face_hi);
    face_lo = face_hi;
  }
  pi0[0] = pi0[1];
  pi0[nz + 1] = pi0[nz];
  for (int k = 0; k <= nz + 1; ++k) {
    const double rt = pow(pi0[k], kCv / kRd) * kP00 / kRd;
    rho0[k] = rt / th0[k] / ((1.0 + kReps * q0[k]) / (1.0 + q0[k]));
  }
}

// FP32 column table from FP64 padded columns (layout documented in Cols)
__global__ void k_build_columns(int nz, double dz, double theta_ref, const double* __restrict__ th0,
                                const double* __restrict__ q0, const double* __restrict__ pi0,
                                const double* __restrict__ rho0, float* __restrict__ tab) {
  const int S = nz + 2;
  float* rho = tab + 0 * S;
  float* rho_face = tab + 1 * S;
  float* rho_face0 = tab + 2 * S;
  float* rho_wext = tab + 3 * S;
  float* theta0 = tab + 4 * S;
  float* qv0 = tab + 5 * S;
  float* trho0 = tab + 6 * S;
  float* d0 = tab + 7 * S;
  float* pic = tab + 8 * S;
  float* dpi0dz = tab + 9 * S;
  float* rho_inv = tab + 10 * S;
  float* rho_w_inv = tab + 11 * S;
  float* rho_wext_inv = tab + 12 * S;
  for (int f = threadIdx.x; f <= nz; f += blockDim.x) {
    if (f < nz) {
      const int L = f + 1;
      rho[f] = (float)rho0[L];
      rho_inv[f] = (float)(1.0 / (double)(float)rho0[L]);
      theta0[f] = (float)th0[L];
      qv0[f] = (float)q0[L];
      trho0[f] = (float)(th0[L] * (1.0 + kReps * q0[L]) / (1.0 + q0[L]));
      d0[f] = (float)(th0[L] - theta_ref);
      pic[f] = (float)pi0[L];
    }
    const double rf = 0.5 * (rho0[f] + rho0[f + 1]);
    rho_face[f] = (float)rf;
    rho_face0[f] = (f == 0 || f == nz) ? 0.f : (float)rf;
    double we;
    if (f == 0)
      we = 1.875 * rho0[1] - 1.25 * rho0[2] + 0.375 * rho0[3];
    else if (f == nz)
      we = 1.875 * rho0[nz] - 1.25 * rho0[nz - 1] + 0.375 * rho0[nz - 2];
    else
      we = rf;
    rho_wext[f] = (float)we;
    rho_wext_inv[f] = (float)(1.0 / (double)(float)we);
    dpi0dz[f] = (float)((pi0[f + 1] - pi0[f]) / dz);
    // the face density of w's advective tendency, formed in FP32 as the kernels form it
    rho_w_inv[f] = (f == 0 || f == nz) ? 0.f : (float)(1.0 / (double)(0.5f * ((float)rho0[f] + (float)rho0[f + 1])));
  }
}

constexpr int RED_THREADS = 256;
constexpr int RED_MAX_BLOCKS = 1024;

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return v;
}

// sums of the budget (kBudgetSums doubles per block, then one final sum each)
__global__ void __launch_bounds__(RED_THREADS) k_budget_partial(Dims d, Phys ph, Cols c, State s,
                                                              const double* __restrict__ rho0_col,
                                                              const double* __restrict__ pi0_col, double theta_ref,
                                                              double* __restrict__ partial) {
  double acc[kBudgetSums] = {0.0, 0.0, 0.0, 0.0, 0.0};
  const long long n = d.cells();
  const double dV = (double)ph.dx * (double)ph.dy * (double)ph.dz;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(t % d.nx);
    const int j = (int)((t / d.nx) % d.ny);
    const int k = (int)(t / ((long long)d.nx * d.ny));
    const double th = theta_ref + (double)s.T[t];
    const double qv = (double)s.q[t];
    const double pi = pi0_col[k + 1] + (double)s.p[t];
    const double p = pow(pi, kCp / kRd) * kP00;  // get_rho, one_step_integration.py:941-947
    const double rho = p / kRd / ((1.0 + kRepsm1 * qv) * (pi * th));
    const double r0 = rho0_col[k + 1];
    const double uc = 0.5 * ((double)s.u[t] + (double)s.u[d.at(wrap(i + 1, d.nx), j, k)]);
    const double vc = 0.5 * ((double)s.v[t] + (double)s.v[d.at(i, wrap(j + 1, d.ny), k)]);
    const double wc = 0.5 * ((double)s.w[t] + (double)s.w[d.at(i, j, k + 1)]);
    const double ke = 0.5 * (uc * uc + vc * vc + wc * wc);
    acc[0] += rho * dV;
    acc[1] += rho * qv * dV;
    acc[2] += r0 * ke * dV;
    acc[3] += r0 * th * dV;
    // total energy: internal (cv T, T = pi theta) + potential (g z at the cell centre) + kinetic
    acc[4] += rho * (kCv * (pi * th) + kG * ((k + 0.5) * (double)ph.dz) + ke) * dV;
  }
  __shared__ double sm[kBudgetSums][RED_THREADS / 32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int m = 0; m < kBudgetSums; ++m) {
    const double v = warp_sum(acc[m]);
    if (lane == 0) sm[m][wid] = v;
  }
  __syncthreads();
  if (wid == 0) {
#pragma unroll
    for (int m = 0; m < kBudgetSums; ++m) {
      double v = lane < RED_THREADS / 32 ? sm[m][lane] : 0.0;
      v = warp_sum(v);
      if (lane == 0) partial[blockIdx.x * kBudgetSums + m] = v;
    }
  }
}

__global__ void k_budget_final(int nblocks, const double* __restrict__ partial, double* __restrict__ out) {
  double acc[kBudgetSums] = {0.0, 0.0, 0.0, 0.0, 0.0};
  for (int b = threadIdx.x; b < nblocks; b += blockDim.x)
#pragma unroll
    for (int m = 0; m < kBudgetSums; ++m) acc[m] += partial[b * kBudgetSums + m];
  __shared__ double sm[kBudgetSums][RED_THREADS / 32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int m = 0; m < kBudgetSums; ++m) {
    const double v = warp_sum(acc[m]);
    if (lane == 0) sm[m][wid] = v;
  }
  __syncthreads();
  if (wid == 0) {
#pragma unroll
    for (int m = 0; m < kBudgetSums; ++m) {
      double v = lane < RED_THREADS / 32 ? sm[m][lane] : 0.0;
      v = warp_sum(v);
      if (lane == 0) out[m] = v;
    }
  }
}

__global__ void k_count_nonfinite(const float* __restrict__ a, long long n, unsigned long long* count) {
  unsigned long long local = 0;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x)
    local += isfinite(a[t]) ? 0ull : 1ull;
  for (int o = 16; o > 0; o >>= 1) local += __shfl_down_sync(0xffffffffu, local, o);
  if ((threadIdx.x & 31) == 0 && local) atomicAdd(count, local);
}

inline int blocks_for(long long n, int threads) {
  long long b = (n + threads - 1) / threads;
  if (b > 4096) b = 4096;
  if (b < 1) b = 1;
  return (int)b;
}

}  // namespace

cudaError_t launch_import_padded(const Dims& d, const void* src, int src_f64, int kind, double offset, float* dst,
                                 cudaStream_t st) {
  const dim3 g((d.nx + TT - 1) / TT, (levels(d, kind) + TT - 1) / TT, d.ny), b(TT, TR);
  if (src_f64)
    k_import_t<double><<<g, b, 0, st>>>(d, (const double*)src, kind, offset, dst);
  else
    k_import_t<float><<<g, b, 0, st>>>(d, (const float*)src, kind, offset, dst);
  return cudaGetLastError();
}

cudaError_t launch_export_padded(const Dims& d, const float* src, int kind, double offset, void* dst, int dst_f64,
                                 cudaStream_t st) {
  int PX, PY, PZ;
  padded_extents(d, kind, PX, PY, PZ);
  const dim3 g((PX + TT - 1) / TT, (PZ + TT - 1) / TT, PY), b(TT, TR);
  if (dst_f64)
    k_export_t<double><<<g, b, 0, st>>>(d, src, kind, offset, (double*)dst);
  else
    k_export_t<float><<<g, b, 0, st>>>(d, src, kind, offset, (float*)dst);
  return cudaGetLastError();
}

cudaError_t launch_export_interior(const Dims& d, const float* src, int kind, double offset, double* dst,
                                   cudaStream_t st) {
  const long long n = (long long)(d.nx + (kind == 1)) * (d.ny + (kind == 2)) * levels(d, kind);
  k_export_interior<<<blocks_for(n, 256), 256, 0, st>>>(d, src, kind, offset, dst);
  return cudaGetLastError();
}

cudaError_t launch_hydrostatic(int nz, double dz, const double* theta0, const double* qv0, double* pi0,
                               double* rho0, cudaStream_t st) {
  k_hydrostatic<<<1, 32, 0, st>>>(nz, dz, theta0, qv0, pi0, rho0);
  return cudaGetLastError();
}

cudaError_t launch_build_columns(int nz, double dz, double theta_ref, const double* theta0, const double* qv0,
                                 const double* pi0, const double* rho0, float* table, cudaStream_t st) {
  k_build_columns<<<1, 256, 0, st>>>(nz, dz, theta_ref, theta0, qv0, pi0, rho0, table);
  return cudaGetLastError();
}

int budget_blocks(const Dims& d) {
  long long b = (d.cells() + RED_THREADS - 1) / RED_THREADS;
  return (int)(b > RED_MAX_BLOCKS ? RED_MAX_BLOCKS : (b < 1 ? 1 : b));
}

cudaError_t launch_budget(const Dims& d, const Phys& ph, const Cols& c, State in, const double* rho0_col,
                          const double* pi0_col, double theta_ref, double* partial, double* out, cudaStream_t st) {
  const int nb = budget_blocks(d);
  k_budget_partial<<<nb, RED_THREADS, 0, st>>>(d, ph, c, in, rho0_col, pi0_col, theta_ref, partial);
  k_budget_final<<<1, RED_THREADS, 0, st>>>(nb, partial, out);
  return cudaGetLastError();
}

cudaError_t launch_count_nonfinite(const float* a, long long n, unsigned long long* count, cudaStream_t st) {
  k_count_nonfinite<<<blocks_for(n, 256), 256, 0, st>>>(a, n, count);
  return cudaGetLastError();
}

}  // namespace lexgb
