// plain.cu — the plain form of the TTSH3D step: one thread per lattice site, the
// reference's stencils evaluated in its arithmetic order, global intermediates.
// It is the FP64 form of the step (and an FP32 form for cross-checks); the fused
// FP32 kernels in fused.cu replace stage1/stage2/div for speed.
//
//   stage1  <- getTempVari_1 + getTempVari_2 (TTSH3D.cu:537-605): mu_0, mu_b, sigma_ab
//   stage2  <- getDtF + getVStar + phi update of getVNew (:608-632, :471-491, :515)
//   div     <- getStream mode 0 for both fields (:664-670), packed as one complex field
//   correct <- getVNew (:494-516), pressures read from the packed complex field
//   stats   <- new FP64 diagnostics (mass, max |div u|, non-finite watchdog)
#include <cstdio>
#include <stdexcept>

#include "common.cuh"
#include "kernels.h"

namespace ttsh {

namespace {

constexpr int BX = 32, BY = 8;

inline void check_launch(const char* what) {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    char buf[256];
    snprintf(buf, sizeof(buf), "%s launch failed: %s", what, cudaGetErrorString(e));
    throw std::runtime_error(buf);
  }
}

inline dim3 site_grid(int N, int n) {
  if ((long)N * n > 65535) throw std::runtime_error("too many instances of this size in one group");
  return dim3((N + BX - 1) / BX, (N + BY - 1) / BY, N * n);
}

template <class T>
__global__ void __launch_bounds__(BX* BY) k_stage1(const InstDev<T>* __restrict__ insts, int par) {
  const int N = insts[0].N;
  const InstDev<T>& I = insts[blockIdx.z / N];
  const int z = blockIdx.z % N;
  const int x = blockIdx.x * BX + threadIdx.x, y = blockIdx.y * BY + threadIdx.y;
  // FP32: this step's maxima of the Poisson source start from zero (k_div records them)
  if (blockIdx.x == 0 && blockIdx.y == 0 && blockIdx.z == 0 && threadIdx.y == 0 && I.wmax)
    for (int i = threadIdx.x; i < 2 * (int)(gridDim.z / N); i += blockDim.x) insts[i >> 1].wmax[i & 1] = 0;
  if (x >= N || y >= N) return;
  Site s;
  s.init(x, y, z, N);
  const Phys<T>& p = I.ph;
  const T* phi = I.phi[par];
  const T ph = phi[s.idx];
  // mu_0 (TTSH3D.cu:567)
  I.mu0[s.idx] = p.aPhi2 * (ph - 3 * ph * ph + 2 * ph * ph * ph) - p.kPhi * st_lap<T>(s.acc(phi), p);
#pragma unroll
  for (int b = 0; b < 3; ++b) {
    Acc<T> F = s.acc<T>(I.P[b]);
    // mu_b (:571-573)
    I.mu[b][s.idx] = ph * I.P[b][s.idx] + p.La2 * st_lap<T>(F, p);
    // sigma_ab = phi * D_a P_b (:587-595; the 1/28 term is an integer-division zero)
    I.sig[0 * 3 + b][s.idx] = ph * st_dx<T>(F, p.c2h);
    I.sig[1 * 3 + b][s.idx] = ph * st_dy<T>(F, p.c2h);
    I.sig[2 * 3 + b][s.idx] = ph * st_dz<T>(F, p.c2h);
  }
}

template <class T>
__global__ void __launch_bounds__(BX* BY) k_stage2(const InstDev<T>* __restrict__ insts, int par) {
  const int N = insts[0].N;
  const InstDev<T>& I = insts[blockIdx.z / N];
  const int z = blockIdx.z % N;
  const int x = blockIdx.x * BX + threadIdx.x, y = blockIdx.y * BY + threadIdx.y;
  if (x >= N || y >= N) return;
  Site s;
  s.init(x, y, z, N);
  const Phys<T>& p = I.ph;
  const int i = s.idx;
  const T* phi = I.phi[par];
  Acc<T> Fphi = s.acc(phi);
  const T dphi[3] = {st_dx<T>(Fphi, p.c2h), st_dy<T>(Fphi, p.c2h), st_dz<T>(Fphi, p.c2h)};
  const T vx = I.U[0][i], vy = I.U[1][i], vz = I.U[2][i];
  const T px = I.P[0][i], py = I.P[1][i], pz = I.P[2][i], ph = phi[i];
  const T P2 = px * px + py * py + pz * pz;
  const T dPhi2 = dphi[0] * dphi[0] + dphi[1] * dphi[1] + dphi[2] * dphi[2];
  const T mu0 = I.mu0[i];
  // getDtF, velocity (TTSH3D.cu:617-621) and getVStar (:480-482)
#pragma unroll
  for (int b = 0; b < 3; ++b) {
    Acc<T> Fv = s.acc<T>(I.U[b]);
    T r = -vx * st_dx<T>(Fv, p.c2h) - vy * st_dy<T>(Fv, p.c2h) - vz * st_dz<T>(Fv, p.c2h) + p.mu * st_lap<T>(Fv, p) +
          mu0 * dphi[b] +
          p.cA * (st_dx<T>(s.acc<T>(I.sig[0 * 3 + b]), p.c2h) + st_dy<T>(s.acc<T>(I.sig[1 * 3 + b]), p.c2h) +
                  st_dz<T>(s.acc<T>(I.sig[2 * 3 + b]), p.c2h));
    if (p.zeta != T(0)) {
      r = r - p.zeta * (st_dx<T>(s.acc_prod<T>(phi, I.P[0], I.P[b]), p.c2h) +
                        st_dy<T>(s.acc_prod<T>(phi, I.P[1], I.P[b]), p.c2h) +
                        st_dz<T>(s.acc_prod<T>(phi, I.P[2], I.P[b]), p.c2h));
    }
    const T u = b == 0 ? vx : (b == 1 ? vy : vz);
    I.Us[par ^ 1][b][i] = u + p.dt * r;
  }
  // getDtF, polarisation (:623-629) and getVStar (:486-488)
  const T pb[3] = {px, py, pz};
#pragma unroll
  for (int b = 0; b < 3; ++b) {
    Acc<T> Fp = s.acc<T>(I.P[b]);
    const T dxp = st_dx<T>(Fp, p.c2h), dyp = st_dy<T>(Fp, p.c2h), dzp = st_dz<T>(Fp, p.c2h);
    T cub;
    if (b == 0) cub = px * px * px + px * py * py + px * pz * pz;
    else if (b == 1) cub = px * py * px + py * py * py + py * pz * pz;
    else cub = px * pz * px + py * pz * py + pz * pz * pz;
    const T Ab = dphi[0] * dphi[b] * px + dphi[1] * dphi[b] * py + dphi[2] * dphi[b] * pz;
    // OP_b + kappa*phi*DP_b are integer-division zeros in the reference (:579-585).
    const T r = -vx * dxp - vy * dyp - vz * dzp - p.alpha * ph * pb[b] - p.beta * P2 * pb[b] +
                p.eta * st_lap<T>(s.acc<T>(I.mu[b]), p) - p.lambda0 * (px * dxp + py * dyp + pz * dzp) -
                p.A * (dPhi2 * cub + sqrt(P2) * Ab);
    I.Ps[par ^ 1][b][i] = pb[b] + p.dt * r;
  }
  // dtphi (:631) and the phi update of getVNew (:515)
  const T dtphi = -vx * dphi[0] - vy * dphi[1] - vz * dphi[2] + p.gamma * (st_lap<T>(s.acc<T>(I.mu0), p));
  I.phi[par ^ 1][i] = ph + p.dt * dtphi;
}

template <class T>
__device__ __forceinline__ T divide_dt(T a, const Phys<T>& p);
template <>
__device__ __forceinline__ double divide_dt<double>(double a, const Phys<double>& p) { return a / p.dt_d; }
template <>
__device__ __forceinline__ float divide_dt<float>(float a, const Phys<float>& p) { return a * p.inv_dt; }

template <class T>
__global__ void __launch_bounds__(BX* BY) k_div(const InstDev<T>* __restrict__ insts, int par) {
  const int N = insts[0].N;
  const InstDev<T>& I = insts[blockIdx.z / N];
  const int z = blockIdx.z % N;
  const int x = blockIdx.x * BX + threadIdx.x, y = blockIdx.y * BY + threadIdx.y;
  if (x >= N || y >= N) return;
  Site s;
  s.init(x, y, z, N);
  const Phys<T>& p = I.ph;
  T d[2];
#pragma unroll
  for (int f = 0; f < 2; ++f) {
    T* const* cur = f == 0 ? I.Us[par ^ 1] : I.Ps[par ^ 1];
    T* const* old = f == 0 ? I.Us[par] : I.Ps[par];
    T a, b, c;
    if (I.stale) {
      a = st_dx<T>(s.acc_stale<T>(cur[0], old[0]), p.c2h);
      b = st_dy<T>(s.acc_stale<T>(cur[1], old[1]), p.c2h);
      c = st_dz<T>(s.acc_stale<T>(cur[2], old[2]), p.c2h);
    } else {
      a = st_dx<T>(s.acc<T>(cur[0]), p.c2h);
      b = st_dy<T>(s.acc<T>(cur[1]), p.c2h);
      c = st_dz<T>(s.acc<T>(cur[2]), p.c2h);
    }
    d[f] = divide_dt<T>(a + b + c, p);  // getStream mode 0 (:666-668)
  }
  typename CxT<T>::type w;
  w.x = d[0];
  w.y = d[1];
  I.W[s.idx] = w;
  if constexpr (sizeof(T) == 4) record_wmax(I.wmax, d[0], d[1]);
}

template <class T>
__global__ void __launch_bounds__(BX* BY) k_correct(const InstDev<T>* __restrict__ insts, int par) {
  const int N = insts[0].N;
  const InstDev<T>& I = insts[blockIdx.z / N];
  const int z = blockIdx.z % N;
  const int x = blockIdx.x * BX + threadIdx.x, y = blockIdx.y * BY + threadIdx.y;
  if (x >= N || y >= N) return;
  Site s;
  s.init(x, y, z, N);
  const Phys<T>& p = I.ph;
  const T* W = reinterpret_cast<const T*>(I.W);
  Acc<T> Fv = s.acc<T>(W, 2), Fp = s.acc<T>(W + 1, 2);
  const int i = s.idx;
  // FP32: the pressures come out of the FFT scaled by powers of two (pow2_norm); undo it exactly
  T du = T(1), dp = T(1);
  if constexpr (sizeof(T) == 4) {
    du = pow2_denorm(I.wmax[0]);
    dp = pow2_denorm(I.wmax[1]);
  }
  // getVNew (TTSH3D.cu:505-511)
  I.U[0][i] = I.Us[par ^ 1][0][i] - p.dt * (st_dx<T>(Fv, p.c2h) * du);
  I.U[1][i] = I.Us[par ^ 1][1][i] - p.dt * (st_dy<T>(Fv, p.c2h) * du);
  I.U[2][i] = I.Us[par ^ 1][2][i] - p.dt * (st_dz<T>(Fv, p.c2h) * du);
  I.P[0][i] = I.Ps[par ^ 1][0][i] - p.dt * (st_dx<T>(Fp, p.c2h) * dp);
  I.P[1][i] = I.Ps[par ^ 1][1][i] - p.dt * (st_dy<T>(Fp, p.c2h) * dp);
  I.P[2][i] = I.Ps[par ^ 1][2][i] - p.dt * (st_dz<T>(Fp, p.c2h) * dp);
}

constexpr int STATS_BLOCKS = 256, STATS_THREADS = 256;

// Diagnostics of the current state (phi[par], u, P): per block, sum(phi), max |D.u|, max |u|, and
// a non-finite count, combined across threads and blocks in FP64 in a fixed order. FP64 fields
// are summed in FP64. FP32 fields are summed by each thread in FP32 with Kahan's compensated
// summation (error of order one rounding of the thread's partial, instead of one per term) and
// only the per-thread partials are combined in FP64: the GPU's FP64 rate is a small fraction of
// its FP32 rate, and an FP64 add per site would cost more than the step's stencils for a mass
// read-back after every step. The maxima are exact in either precision.
template <class T>
struct MassAcc;
template <>
struct MassAcc<double> {
  double s = 0;
  __device__ __forceinline__ void add(double v) { s += v; }
  __device__ __forceinline__ double total() const { return s; }
};
template <>
struct MassAcc<float> {
  float s = 0.f, c = 0.f;  // Kahan: c carries the low part lost by the last addition
  __device__ __forceinline__ void add(float v) {
    const float y = v - c;
    const float t = s + y;
    c = (t - s) - y;
    s = t;
  }
  __device__ __forceinline__ double total() const { return (double)s - (double)c; }
};

// Block reduction of the four per-thread diagnostics (fixed order) into the block's partials.
template <class T>
__device__ __forceinline__ void stats_finish(const InstDev<T>& I, double sum, double mdiv, double mu, double bad) {
  __shared__ double sh[4][STATS_THREADS / 32];
  for (int o = 16; o > 0; o >>= 1) {
    sum += __shfl_down_sync(0xffffffffu, sum, o);
    mdiv = fmax(mdiv, __shfl_down_sync(0xffffffffu, mdiv, o));
    mu = fmax(mu, __shfl_down_sync(0xffffffffu, mu, o));
    bad += __shfl_down_sync(0xffffffffu, bad, o);
  }
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) { sh[0][w] = sum; sh[1][w] = mdiv; sh[2][w] = mu; sh[3][w] = bad; }
  __syncthreads();
  if (threadIdx.x == 0) {
    double a = 0, b = 0, c = 0, e = 0;
    for (int k = 0; k < STATS_THREADS / 32; ++k) {
      a += sh[0][k]; b = fmax(b, sh[1][k]); c = fmax(c, sh[2][k]); e += sh[3][k];
    }
    double* out = I.red + 4 * blockIdx.x;
    out[0] = a; out[1] = b; out[2] = c; out[3] = e;
  }
}

// 16-byte vectors of T (the mass-only pass reads phi with them).
template <class T> struct Vec16;
template <> struct Vec16<float> { typedef float4 type; };
template <> struct Vec16<double> { typedef double2 type; };

// Sum of phi over this thread's share of the sites (fixed order) and the count of non-finite
// values: 16-byte loads, four in flight per thread, and one compensated accumulator per vector
// lane, so that the pass streams phi at HBM speed (one 4-byte load per thread in flight had kept
// it at a few hundred GB/s). Both diagnostics modes take the mass from here, so they agree.
template <class T>
__device__ __forceinline__ double mass_pass(const T* __restrict__ phi, long n, int& badn) {
  typedef typename Vec16<T>::type V;
  constexpr int W = (int)(sizeof(V) / sizeof(T));
  const long nv = n / W, stride = (long)gridDim.x * blockDim.x;
  const V* __restrict__ pv = reinterpret_cast<const V*>(phi);
  MassAcc<T> lane[W];
  auto take = [&](const V& v) {
    const T* e = reinterpret_cast<const T*>(&v);
#pragma unroll
    for (int c = 0; c < W; ++c) {
      lane[c].add(e[c]);
      badn += isfinite(e[c]) ? 0 : 1;
    }
  };
  long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  for (; i + 3 * stride < nv; i += 4 * stride) {
    V v[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) v[u] = pv[i + u * stride];
#pragma unroll
    for (int u = 0; u < 4; ++u) take(v[u]);
  }
  for (; i < nv; i += stride) take(pv[i]);
  for (long j = nv * W + (long)blockIdx.x * blockDim.x + threadIdx.x; j < n; j += stride) {
    lane[0].add(phi[j]);
    badn += isfinite(phi[j]) ? 0 : 1;
  }
  double tot = 0;
#pragma unroll
  for (int c = 0; c < W; ++c) tot += lane[c].total();
  return tot;
}

template <class T, bool FULL>
__global__ void __launch_bounds__(STATS_THREADS) k_stats(const InstDev<T>* __restrict__ insts, int par) {
  const InstDev<T>& I = insts[blockIdx.y];
  const int N = I.N;
  const long n = (long)N * N * N;
  int badn = 0;
  const double mass = mass_pass<T>(I.phi[par], n, badn);
  T mdivT = 0, muT = 0;
  if constexpr (FULL) {
    // max |D.u|, max |u| and the non-finite values of u and P
    const Phys<T>& p = I.ph;
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
      const int x = (int)(i % N), y = (int)((i / N) % N), z = (int)(i / ((long)N * N));
      Site s;
      s.init(x, y, z, N);
      const T d = st_dx<T>(s.acc<T>(I.U[0]), p.c2h) + st_dy<T>(s.acc<T>(I.U[1]), p.c2h) + st_dz<T>(s.acc<T>(I.U[2]), p.c2h);
      mdivT = fmax(mdivT, fabs(d));
      for (int b = 0; b < 3; ++b) {
        const T u = I.U[b][i], q = I.P[b][i];
        muT = fmax(muT, fabs(u));
        if (!isfinite(u) || !isfinite(q)) badn += 1;
      }
    }
  }
  stats_finish<T>(I, mass, (double)mdivT, (double)muT, (double)badn);
}

}  // namespace

int stats_partials_per_instance(int) { return STATS_BLOCKS; }

template <class T>
void launch_stage1(const Group<T>& g, int par, cudaStream_t st) {
  k_stage1<T><<<site_grid(g.N, g.n), dim3(BX, BY), 0, st>>>(g.d_inst, par);
  check_launch("stage1");
}
template <class T>
void launch_stage2(const Group<T>& g, int par, cudaStream_t st) {
  k_stage2<T><<<site_grid(g.N, g.n), dim3(BX, BY), 0, st>>>(g.d_inst, par);
  check_launch("stage2");
}
template <class T>
void launch_div(const Group<T>& g, int par, cudaStream_t st) {
  k_div<T><<<site_grid(g.N, g.n), dim3(BX, BY), 0, st>>>(g.d_inst, par);
  check_launch("div");
}
template <class T>
void launch_correct(const Group<T>& g, int par, cudaStream_t st) {
  k_correct<T><<<site_grid(g.N, g.n), dim3(BX, BY), 0, st>>>(g.d_inst, par);
  check_launch("correct");
}
template <class T>
int launch_stats(const Group<T>& g, int par, cudaStream_t st, bool full) {
  if (full) k_stats<T, true><<<dim3(STATS_BLOCKS, g.n), STATS_THREADS, 0, st>>>(g.d_inst, par);
  else k_stats<T, false><<<dim3(STATS_BLOCKS, g.n), STATS_THREADS, 0, st>>>(g.d_inst, par);
  check_launch("stats");
  return STATS_BLOCKS;
}

#define INST(T)                                                          \
  template void launch_stage1<T>(const Group<T>&, int, cudaStream_t);   \
  template void launch_stage2<T>(const Group<T>&, int, cudaStream_t);   \
  template void launch_div<T>(const Group<T>&, int, cudaStream_t);      \
  template void launch_correct<T>(const Group<T>&, int, cudaStream_t);  \
  template int launch_stats<T>(const Group<T>&, int, cudaStream_t, bool);
INST(float)
INST(double)
#undef INST

}  // namespace ttsh
