// common.cuh — shared device types of libttsh: per-droplet descriptors and the
// reference-order stencils of TTSH3D.cu (d1{x,y,z}CO2I3D, laplaceCO2I3D, :3280-3343).
#pragma once
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>

namespace ttsh {

template <class T> struct CxT;
template <> struct CxT<float> { typedef float2 type; };
template <> struct CxT<double> { typedef double2 type; };

// Physics constants of one droplet, in the arithmetic type T. The stencil
// prefactors are formed on the host in FP64, as the reference forms them on
// the device in FP64 (1.0/(2.0*h), 1.0/(12*h*h), 2.0/(3*h*h), 14.0/(3*h*h)).
template <class T>
struct Phys {
  T h, dt, inv_dt;
  T mu, cA, alpha, beta, eta, La2, kappa, lambda0, aPhi2, kPhi, gamma, A, zeta;
  T c2h;           // 1/(2h)
  T cl12, cl23, cl143;  // 1/(12h^2), 2/(3h^2), 14/(3h^2)
  T clz;           // 1/h^2 (the fused form's shift-invariant Laplacian)
  T invN3;         // 1/N^3 (FP32 path); FP64 path divides by (double)N^3 as getStream mode 2
  double dt_d;     // dt in FP64 (divisor of getStream mode 0 in the FP64 path)
};

// Per-droplet device descriptor. Field arrays are unpadded N^3, x fastest.
// Ping-pong pairs are indexed by the step parity `par`: the step reads
// phi[par], Us[par], Ps[par] and writes phi[par^1], Us[par^1], Ps[par^1].
template <class T>
struct InstDev {
  typedef typename CxT<T>::type C;
  int N, stale, k2mode, nstages;
  int radix[16];
  Phys<T> ph;
  T* phi[2];
  T* P[3];
  T* U[3];
  T* Us[2][3];
  T* Ps[2][3];
  C* W;               // N^3 complex: (div u* + i div P*)/dt -> (p_v + i p_p)
  T* phic;            // fused form: compensation of the phi update (the low part lost to rounding)
  int* wmax;          // FP32 forms: max |Re W|, max |Im W| of this step's Poisson source (float bits,
                      // non-negative floats order as ints); null in the FP64 form
  // Fused FP32 form only (null elsewhere): u and the u*, P* ping-pong stored compensated, the
  // FP32 value plus, in bf16, the part of the exact value its rounding dropped; u*, P* as pairs
  // (u*_b, P*_b), which the divergence and the correction read together
  __nv_bfloat16* lo[3];            // u
  float2* star[2][3];              // (u*_b, P*_b) of parity q (Us, Ps are null in the fused form)
  __nv_bfloat162* starlo[2][3];    // their compensations
  int* smax;                       // max |u*|, max |P*| of this step (float bits): the divergence's grid
  T* mu0;             // plain-form intermediates
  T* mu[3];
  T* sig[9];          // sig[a*3+b] = phi * D_a P_b
  const C* tw;        // tw[k] = exp(-2 pi i k / N), k < N
  const double* kval; // k(m), FP64 (continuous wavenumber of initPoissonSolver)
  const T* k2t;       // k(m)^2 rounded to T
  const T* St;        // sin(k h)/h
  const T* Ct;        // (2 + cos(k h))/3
  double* red;        // FP64 reduction partials
};

__host__ __device__ inline int wrapi(int a, int N) { return a < 0 ? a + N : (a >= N ? a - N : a); }

// The packed Poisson source W = D.u*/dt + i D.P*/dt of the FP32 forms is transformed as one
// complex field. Its two parts can differ in size by orders of magnitude (the divergence of the
// polarisation is large while P is far from solenoidal), and the rounding of every complex
// operation is relative to the larger part: in FP32 that error would swamp the smaller part (a
// relative error of 1e-4 in p_v when |D.P*| is 500 x |D.u*|). So the first forward pass scales
// each part by the power of two that brings its maximum into [1, 2), and the correction (and the
// read-back of the pressures) undoes it; powers of two scale exactly, so only the balance changes.
// Scale for a maximum given as float bits (0: no scaling).
__host__ __device__ inline float pow2_norm(int mbits) {
  if (mbits <= 0) return 1.f;
  int e = ((mbits >> 23) & 0xff) - 127;
  e = e < -125 ? -125 : (e > 125 ? 125 : e);
  const unsigned bits = (unsigned)(127 - e) << 23;
  float s;
  memcpy(&s, &bits, sizeof s);
  return s;
}
// Its inverse, exact.
__host__ __device__ inline float pow2_denorm(int mbits) {
  if (mbits <= 0) return 1.f;
  int e = ((mbits >> 23) & 0xff) - 127;
  e = e < -125 ? -125 : (e > 125 ? 125 : e);
  const unsigned bits = (unsigned)(127 + e) << 23;
  float s;
  memcpy(&s, &bits, sizeof s);
  return s;
}
// Warp-aggregated record of two maxima |a|, |b| (float bits) into dst[0..1] (the Poisson source's
// parts, the provisional fields); any subset of a warp's lanes may call it.
__device__ __forceinline__ void record_wmax(int* wmax, float ax, float ay) {
  const unsigned act = __activemask();
  const unsigned mx = __reduce_max_sync(act, __float_as_uint(fabsf(ax)));
  const unsigned my = __reduce_max_sync(act, __float_as_uint(fabsf(ay)));
  unsigned lane;
  asm("mov.u32 %0, %%laneid;" : "=r"(lane));
  if (lane == (unsigned)(__ffs(act) - 1)) {
    atomicMax(wmax, (int)mx);
    atomicMax(wmax + 1, (int)my);
  }
}

// Accessor of a scalar field around (x,y,z) with periodic wrap.
template <class T>
struct Acc {
  const T* __restrict__ f;
  int xo[3], yo[3], zo[3];
  int stride;  // 1 for real arrays, 2 for one component of an interleaved complex array
  __device__ __forceinline__ T operator()(int dx, int dy, int dz) const {
    return __ldg(f + (size_t)stride * (zo[dz + 1] + yo[dy + 1] + xo[dx + 1]));
  }
};

// Accessor whose wrapped neighbours come from `old` (quirk Q2 of the reference:
// the halo of u*/P* is refreshed at the start of getRHS, TTSH3D.cu:369-371 and
// :405-407, before getVStar rewrites the interior, :471-491).
template <class T>
struct AccStale {
  const T* __restrict__ f;
  const T* __restrict__ old;
  int xo[3], yo[3], zo[3];
  bool wx[3], wy[3], wz[3];
  __device__ __forceinline__ T operator()(int dx, int dy, int dz) const {
    const T* p = (wx[dx + 1] | wy[dy + 1] | wz[dz + 1]) ? old : f;
    return __ldg(p + zo[dz + 1] + yo[dy + 1] + xo[dx + 1]);
  }
};

// Accessor of the pointwise product phi * Pa * Pb (build-defined active stress).
template <class T>
struct AccProd {
  const T* __restrict__ phi;
  const T* __restrict__ pa;
  const T* __restrict__ pb;
  int xo[3], yo[3], zo[3];
  __device__ __forceinline__ T operator()(int dx, int dy, int dz) const {
    int i = zo[dz + 1] + yo[dy + 1] + xo[dx + 1];
    return __ldg(phi + i) * __ldg(pa + i) * __ldg(pb + i);
  }
};

struct Site {
  int xo[3], yo[3], zo[3];
  bool wx[3], wy[3], wz[3];
  int idx;
  __device__ __forceinline__ void init(int x, int y, int z, int N) {
    int NN = N * N;
    xo[0] = wrapi(x - 1, N); xo[1] = x; xo[2] = wrapi(x + 1, N);
    yo[0] = wrapi(y - 1, N) * N; yo[1] = y * N; yo[2] = wrapi(y + 1, N) * N;
    zo[0] = wrapi(z - 1, N) * NN; zo[1] = z * NN; zo[2] = wrapi(z + 1, N) * NN;
    wx[0] = x == 0; wx[1] = false; wx[2] = x == N - 1;
    wy[0] = y == 0; wy[1] = false; wy[2] = y == N - 1;
    wz[0] = z == 0; wz[1] = false; wz[2] = z == N - 1;
    idx = z * NN + y * N + x;
  }
  template <class T>
  __device__ __forceinline__ Acc<T> acc(const T* f, int stride = 1) const {
    Acc<T> a;
    a.f = f;
    a.stride = stride;
#pragma unroll
    for (int i = 0; i < 3; ++i) { a.xo[i] = xo[i]; a.yo[i] = yo[i]; a.zo[i] = zo[i]; }
    return a;
  }
  template <class T>
  __device__ __forceinline__ AccStale<T> acc_stale(const T* f, const T* old) const {
    AccStale<T> a;
    a.f = f;
    a.old = old;
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      a.xo[i] = xo[i]; a.yo[i] = yo[i]; a.zo[i] = zo[i];
      a.wx[i] = wx[i]; a.wy[i] = wy[i]; a.wz[i] = wz[i];
    }
    return a;
  }
  template <class T>
  __device__ __forceinline__ AccProd<T> acc_prod(const T* phi, const T* pa, const T* pb) const {
    AccProd<T> a;
    a.phi = phi; a.pa = pa; a.pb = pb;
#pragma unroll
    for (int i = 0; i < 3; ++i) { a.xo[i] = xo[i]; a.yo[i] = yo[i]; a.zo[i] = zo[i]; }
    return a;
  }
};

// The 27-point first derivatives and the 15-point Laplacian, with the
// reference's neighbour order and constants (TTSH3D.cu:3280-3343).
template <class T, class A>
__device__ __forceinline__ T st_dx(const A& F, T c2h) {
  return c2h * (T(16.0 / 36) * (F(1, 0, 0) - F(-1, 0, 0)) +
                T(4.0 / 36) * (F(1, 0, 1) + F(1, 0, -1) + F(1, 1, 0) + F(1, -1, 0) - F(-1, 0, 1) - F(-1, 0, -1) -
                               F(-1, 1, 0) - F(-1, -1, 0)) +
                T(1.0 / 36) * (F(1, 1, 1) + F(1, -1, 1) + F(1, 1, -1) + F(1, -1, -1) - F(-1, 1, 1) - F(-1, -1, 1) -
                               F(-1, 1, -1) - F(-1, -1, -1)));
}
template <class T, class A>
__device__ __forceinline__ T st_dy(const A& F, T c2h) {
  return c2h * (T(16.0 / 36) * (F(0, 1, 0) - F(0, -1, 0)) +
                T(4.0 / 36) * (F(0, 1, 1) + F(0, 1, -1) + F(1, 1, 0) + F(-1, 1, 0) - F(0, -1, 1) - F(0, -1, -1) -
                               F(1, -1, 0) - F(-1, -1, 0)) +
                T(1.0 / 36) * (F(1, 1, 1) + F(-1, 1, 1) + F(1, 1, -1) + F(-1, 1, -1) - F(1, -1, 1) - F(-1, -1, 1) -
                               F(1, -1, -1) - F(-1, -1, -1)));
}
template <class T, class A>
__device__ __forceinline__ T st_dz(const A& F, T c2h) {
  return c2h * (T(16.0 / 36) * (F(0, 0, 1) - F(0, 0, -1)) +
                T(4.0 / 36) * (F(1, 0, 1) + F(-1, 0, 1) + F(0, 1, 1) + F(0, -1, 1) - F(1, 0, -1) - F(-1, 0, -1) -
                               F(0, 1, -1) - F(0, -1, -1)) +
                T(1.0 / 36) * (F(1, 1, 1) + F(1, -1, 1) + F(-1, 1, 1) + F(-1, -1, 1) - F(1, 1, -1) - F(1, -1, -1) -
                               F(-1, 1, -1) - F(-1, -1, -1)));
}
template <class T, class A>
__device__ __forceinline__ T st_lap(const A& F, const Phys<T>& p) {
  return p.cl12 * (F(1, 1, -1) + F(1, -1, -1) + F(-1, 1, -1) + F(-1, -1, -1) + F(1, 1, 1) + F(1, -1, 1) +
                   F(-1, 1, 1) + F(-1, -1, 1)) +
         p.cl23 * (F(0, 0, -1) + F(0, 0, 1) + F(-1, 0, 0) + F(1, 0, 0) + F(0, -1, 0) + F(0, 1, 0)) -
         p.cl143 * F(0, 0, 0);
}

}  // namespace ttsh
