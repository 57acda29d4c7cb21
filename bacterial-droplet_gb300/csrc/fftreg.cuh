// fftreg.cuh — register-resident two-level FFT passes (the fast path of fft.cu's passes).
//
// A line of length N = N1*N2 is transformed as in the "four-step" factorisation:
//   Y[k1][n2] = DFT_N1 over n1 of x[N2*n1 + n2]                 (thread n2 holds x[N2*n1+n2])
//   X[k1 + N1*k2] = DFT_N2 over n2 of w_N^(n2*k1) * Y[k1][n2]    (after one shared-memory transpose)
// and the inverse runs the same steps backwards. Each thread keeps its N1 (or N2) values in
// registers; small DFTs are expanded at compile time by mixed-radix decimation in time
// (radix 4, 2, 3, 5), with twiddles read from the FP64-built table exp(-2 pi i k / N).
// The z pass goes forward, applies the Poisson multiplier and goes back without leaving the
// CTA: two shared-memory transposes for the whole forward-divide-inverse sequence.
#pragma once
#include "common.cuh"

namespace ttsh {
namespace fftreg {

template <class C>
__device__ __forceinline__ C cmul(C a, C b) {
  C r;
  r.x = a.x * b.x - a.y * b.y;
  r.y = a.x * b.y + a.y * b.x;
  return r;
}
template <class C>
__device__ __forceinline__ C cadd(C a, C b) { C r; r.x = a.x + b.x; r.y = a.y + b.y; return r; }
template <class C>
__device__ __forceinline__ C csub(C a, C b) { C r; r.x = a.x - b.x; r.y = a.y - b.y; return r; }
// FP32: one packed instruction (add/sub .f32x2: two IEEE FP32 operations, round to nearest, the
// results of the two scalar ones) per complex add or subtract.
__device__ __forceinline__ float2 cadd(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 csub(float2 a, float2 b) {
  float2 d;
  asm("sub.rn.f32x2 %0, %1, %2;"
      : "=l"(*reinterpret_cast<unsigned long long*>(&d))
      : "l"(*reinterpret_cast<const unsigned long long*>(&a)), "l"(*reinterpret_cast<const unsigned long long*>(&b)));
  return d;
}
// exp(-+2 pi i k / N) from the table; conjugate for the inverse.
template <class C, bool INV>
__device__ __forceinline__ C tw(const C* t, int k) {
  C w = __ldg(t + k);
  if (INV) w.y = -w.y;
  return w;
}

constexpr int first_radix(int L) { return L % 4 == 0 ? 4 : (L % 2 == 0 ? 2 : (L % 3 == 0 ? 3 : 5)); }

// exp(-2 pi i k / NF) from the __constant__ copy of the size-NF table (defined per size by
// fftreg_impl.cuh): with a compile-time k it is a constant-bank operand, not a load.
template <class C, int NF>
__device__ C ctw(int k);

// twiddle k of the DFT's table: the __constant__ copy when the line length NF is known (NF > 0),
// else the table in global memory
template <class C, bool INV, int NF>
__device__ __forceinline__ C twx(const C* t, int k) {
  if constexpr (NF > 0) {
    C w = ctw<C, NF>(k);
    if (INV) w.y = -w.y;
    return w;
  } else {
    return tw<C, INV>(t, k);
  }
}

// In-place DFT of v[0..L) (natural order in and out). `step` = N / L, so that w_L^m = tab[m*step].
// NF: the table's length when it has a __constant__ copy (0: read `tab`).
template <class C, int L, bool INV, int NF = 0>
struct Dft {
  static __device__ __forceinline__ void run(C* v, const C* tab, int step) {
    constexpr int R = first_radix(L);
    constexpr int M = L / R;
    if constexpr (L == 1) {
      return;
    } else if constexpr (L == 2) {
      C a = v[0], b = v[1];
      v[0] = cadd(a, b);
      v[1] = csub(a, b);
    } else if constexpr (L == 4) {
      C a = cadd(v[0], v[2]), b = csub(v[0], v[2]), c = cadd(v[1], v[3]), d = csub(v[1], v[3]);
      C dd;
      if (INV) { dd.x = -d.y; dd.y = d.x; } else { dd.x = d.y; dd.y = -d.x; }
      v[0] = cadd(a, c);
      v[2] = csub(a, c);
      v[1] = cadd(b, dd);
      v[3] = csub(b, dd);
    } else if constexpr (L == 3 || L == 5) {
      C o[L];
#pragma unroll
      for (int q = 0; q < L; ++q) {
        C acc = v[0];
#pragma unroll
        for (int r = 1; r < L; ++r) acc = cadd(acc, cmul(v[r], twx<C, INV, NF>(tab, ((q * r) % L) * step)));
        o[q] = acc;
      }
#pragma unroll
      for (int q = 0; q < L; ++q) v[q] = o[q];
    } else {
      // decimation in time: R sub-sequences v[r + R*m], each a DFT of length M
      C u[R][M];
#pragma unroll
      for (int r = 0; r < R; ++r) {
#pragma unroll
        for (int m = 0; m < M; ++m) u[r][m] = v[r + R * m];
        Dft<C, M, INV, NF>::run(u[r], tab, step * R);
      }
#pragma unroll
      for (int k0 = 0; k0 < M; ++k0) {
        C t[R];
#pragma unroll
        for (int r = 0; r < R; ++r) t[r] = (r > 0 && k0 > 0) ? cmul(u[r][k0], twx<C, INV, NF>(tab, r * k0 * step)) : u[r][k0];
        Dft<C, R, INV, NF>::run(t, tab, step * M);
#pragma unroll
        for (int k1 = 0; k1 < R; ++k1) v[k0 + M * k1] = t[k1];
      }
    }
  }
};

// -F / k^2 of getStream mode 1 (:672-683) with k2 from initPoissonSolver (:1088-1124).
__device__ __forceinline__ double2 poisson_mul(double2 v, const InstDev<double>& I, int x, int y, int z) {
  double k2;
  if (I.k2mode == 0) {
    const double kx = I.kval[x], ky = I.kval[y], kz = I.kval[z];
    // the host's kx*kx + ky*ky + kz*kz, without contraction
    k2 = __dadd_rn(__dadd_rn(__dmul_rn(kx, kx), __dmul_rn(ky, ky)), __dmul_rn(kz, kz));
    if ((x | y | z) == 0) k2 = 1;  // k2[0] = 1 (:1120)
  } else {
    const double Kx = I.St[x] * I.Ct[y] * I.Ct[z], Ky = I.Ct[x] * I.St[y] * I.Ct[z], Kz = I.Ct[x] * I.Ct[y] * I.St[z];
    k2 = Kx * Kx + Ky * Ky + Kz * Kz;
    if (k2 < 1e-8 / ((double)I.ph.h * (double)I.ph.h)) return make_double2(0.0, 0.0);
  }
  return make_double2(-v.x / k2, -v.y / k2);
}
__device__ __forceinline__ float2 poisson_mul(float2 v, const InstDev<float>& I, int x, int y, int z) {
  float k2;
  if (I.k2mode == 0) {
    k2 = I.k2t[x] + I.k2t[y] + I.k2t[z];
    if ((x | y | z) == 0) k2 = 1.f;
  } else {
    const float Kx = I.St[x] * I.Ct[y] * I.Ct[z], Ky = I.Ct[x] * I.St[y] * I.Ct[z], Kz = I.Ct[x] * I.Ct[y] * I.St[z];
    k2 = Kx * Kx + Ky * Ky + Kz * Kz;
    if (k2 < 1e-8f / (I.ph.h * I.ph.h)) return make_float2(0.f, 0.f);
  }
  // the correctly rounded reciprocal: the value of -1.f / k2 without a full division routine
  const float f = -__frcp_rn(k2);
  return make_float2(v.x * f, v.y * f);
}

__device__ __forceinline__ double2 scale_n3(double2 v, const InstDev<double>& I) {
  const double n3 = (double)(I.N * I.N * I.N);
  return make_double2(v.x / n3, v.y / n3);
}
__device__ __forceinline__ float2 scale_n3(float2 v, const InstDev<float>& I) {
  return make_float2(v.x * I.ph.invN3, v.y * I.ph.invN3);
}

}  // namespace fftreg
}  // namespace ttsh
