// fftreg_impl.cuh — the register-resident FFT pass kernel and its size table, instantiated for
// one arithmetic type by fftreg_f32.cu / fftreg_f64.cu (two translation units build in parallel).
#pragma once
#include <stdexcept>
#include <string>

#include "common.cuh"
#include "fftreg.cuh"
#include "kernels.h"

namespace ttsh {
namespace fftreg {

// Lines per CTA: adjacent in x for the y and z passes (coalesced 128-byte rows), consecutive
// rows for the x pass.
template <int N>
constexpr int lines_per_cta() { return N % 16 == 0 ? 16 : (N % 8 == 0 ? 8 : (N % 4 == 0 ? 4 : (N % 2 == 0 ? 2 : 1))); }

template <class T, int N1, int N2>
constexpr size_t smem_bytes(int axis) {
  typedef typename CxT<T>::type C;
  constexpr int LB = lines_per_cta<N1 * N2>();
  return axis == 0 ? (size_t)LB * N1 * (N2 + 1) * sizeof(C) : (size_t)N1 * N2 * LB * sizeof(C);
}

// PASS: 0 forward x, 1 forward y, 2 forward z + Poisson multiplier + inverse z, 3 inverse y,
// 4 inverse x scaled by 1/N^3. One call transforms line group g of the pass (LB lines) with the
// CTA's threads; S is the CTA's shared memory.
template <class T, int N1, int N2, int PASS>
__device__ __forceinline__ void fft_lines(const InstDev<T>& I, int g, typename CxT<T>::type* S) {
  typedef typename CxT<T>::type C;
  constexpr int N = N1 * N2;
  constexpr int LB = lines_per_cta<N>();
  constexpr int OW = N1 / N2;  // k1 rows owned by each thread in the second step
  constexpr int axis = (PASS == 0 || PASS == 4) ? 0 : ((PASS == 1 || PASS == 3) ? 1 : 2);
  C* __restrict__ W = I.W;
  const C* tab = I.tw;
  const size_t NN = (size_t)N * N;
  const int t = threadIdx.x;
  int l, j;
  if (axis == 0) { j = t % N2; l = t / N2; } else { l = t % LB; j = t / LB; }
  size_t base, stride;
  int xl = 0, yl = 0;
  {
    if (axis == 0) {
      base = ((size_t)g * LB + l) * N;
      stride = 1;
    } else {
      constexpr int ng = N / LB;
      const int outer = g / ng;
      xl = (g - outer * ng) * LB + l;
      if (axis == 1) { base = (size_t)outer * NN + xl; stride = N; }
      else { base = (size_t)outer * N + xl; stride = NN; yl = outer; }
    }
  }
  auto sidx = [&](int k1, int n2) -> int {
    return axis == 0 ? (l * (N1 * (N2 + 1)) + k1 * (N2 + 1) + n2) : ((k1 * N2 + n2) * LB + l);
  };
  constexpr bool FWD_FIRST = (PASS == 0 || PASS == 1 || PASS == 2);
  if constexpr (FWD_FIRST) {
    // first step: thread n2 = j transforms x[N2*n1 + j], n1 < N1
    C v[N1];
#pragma unroll
    for (int n1 = 0; n1 < N1; ++n1) v[n1] = W[base + (size_t)(N2 * n1 + j) * stride];
    Dft<C, N1, false>::run(v, tab, N2);
#pragma unroll
    for (int k1 = 0; k1 < N1; ++k1) S[sidx(k1, j)] = (k1 > 0 && j > 0) ? cmul(v[k1], tw<C, false>(tab, j * k1)) : v[k1];
    __syncthreads();
#pragma unroll
    for (int o = 0; o < OW; ++o) {
      const int k1 = j + N2 * o;
      C u[N2];
#pragma unroll
      for (int n2 = 0; n2 < N2; ++n2) u[n2] = S[sidx(k1, n2)];
      Dft<C, N2, false>::run(u, tab, N1);
      if constexpr (PASS == 2) {
        // spectrum element z = k1 + N1*k2 of the line (x = xl, y = yl): multiply, go back
#pragma unroll
        for (int k2 = 0; k2 < N2; ++k2) u[k2] = poisson_mul(u[k2], I, xl, yl, k1 + N1 * k2);
        Dft<C, N2, true>::run(u, tab, N1);
#pragma unroll
        for (int n2 = 0; n2 < N2; ++n2) S[sidx(k1, n2)] = (n2 > 0 && k1 > 0) ? cmul(u[n2], tw<C, true>(tab, n2 * k1)) : u[n2];
      } else {
#pragma unroll
        for (int k2 = 0; k2 < N2; ++k2) W[base + (size_t)(k1 + N1 * k2) * stride] = u[k2];
      }
    }
    if constexpr (PASS == 2) {
      __syncthreads();
      C x[N1];
#pragma unroll
      for (int k1 = 0; k1 < N1; ++k1) x[k1] = S[sidx(k1, j)];
      Dft<C, N1, true>::run(x, tab, N2);
#pragma unroll
      for (int n1 = 0; n1 < N1; ++n1) W[base + (size_t)(N2 * n1 + j) * stride] = x[n1];
    }
  } else {
    // inverse: rows k1 (owned) hold X[k1 + N1*k2]; inverse DFT over k2, twiddle, transpose, inverse over k1
#pragma unroll
    for (int o = 0; o < OW; ++o) {
      const int k1 = j + N2 * o;
      C u[N2];
#pragma unroll
      for (int k2 = 0; k2 < N2; ++k2) u[k2] = W[base + (size_t)(k1 + N1 * k2) * stride];
      Dft<C, N2, true>::run(u, tab, N1);
#pragma unroll
      for (int n2 = 0; n2 < N2; ++n2) S[sidx(k1, n2)] = (n2 > 0 && k1 > 0) ? cmul(u[n2], tw<C, true>(tab, n2 * k1)) : u[n2];
    }
    __syncthreads();
    C x[N1];
#pragma unroll
    for (int k1 = 0; k1 < N1; ++k1) x[k1] = S[sidx(k1, j)];
    Dft<C, N1, true>::run(x, tab, N2);
#pragma unroll
    for (int n1 = 0; n1 < N1; ++n1) {
      C v = x[n1];
      if constexpr (PASS == 4) v = scale_n3(v, I);
      W[base + (size_t)(N2 * n1 + j) * stride] = v;
    }
  }
}

// Minimum CTAs per SM. The FP32 z pass (forward, divide, inverse) trades a few
// spilled registers for occupancy; measured at 256^3 (2 droplets): 4 CTAs 0.164 ms, 3 CTAs
// 0.176 ms, 2 CTAs 0.196 ms per step. Other sizes keep the settings they were measured with.
template <class T, int N, int PASS>
constexpr int fftr_min_blocks() {
  return (sizeof(T) == 4 && PASS == 2) ? (N == 256 ? 4 : (N > 256 ? 3 : 1)) : 1;
}

template <class T, int N1, int N2, int PASS>
__global__ void __launch_bounds__(lines_per_cta<N1 * N2>() * N2, fftr_min_blocks<T, N1 * N2, PASS>()) k_fftr(const InstDev<T>* __restrict__ insts) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  fft_lines<T, N1, N2, PASS>(insts[blockIdx.y], blockIdx.x, reinterpret_cast<typename CxT<T>::type*>(smem_raw));
}

// Both in-plane axes of the z-planes, one plane per thread-block cluster of PC CTAs: DIR 0
// forward x then forward y, DIR 1 inverse y then inverse x (scaled). Each CTA of the cluster
// takes every PC-th line group of the first axis, the cluster barrier (release / acquire at
// cluster scope) makes the whole plane's results visible to all of its CTAs, then each takes
// every PC-th line group of the second axis. The plane's intermediate (N^2 complex values) is
// written and read back a few microseconds apart, so it stays in L2 instead of making an HBM
// round trip between two separate passes over the whole volume.
template <int N>
constexpr int plane_parts() {
  constexpr int NG = N / lines_per_cta<N>();
  return NG % 4 == 0 ? 4 : (NG % 2 == 0 ? 2 : (NG % 3 == 0 ? 3 : 1));
}


__device__ __forceinline__ void cluster_sync_all() {
  asm volatile("barrier.cluster.arrive.release.aligned;\n" ::: "memory");
  asm volatile("barrier.cluster.wait.acquire.aligned;\n" ::: "memory");
}

template <class T, int N1, int N2, int DIR>
__device__ __forceinline__ void plane_body(const InstDev<T>* __restrict__ insts) {
  typedef typename CxT<T>::type C;
  constexpr int N = N1 * N2;
  constexpr int NG = N / lines_per_cta<N>();  // line groups of one axis within a plane
  constexpr int PC = plane_parts<N>();
  static_assert(NG % PC == 0, "the cluster splits a plane's line groups evenly");
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C* S = reinterpret_cast<C*>(smem_raw);
  const InstDev<T>& I = insts[blockIdx.y];
  const int z = blockIdx.x / PC, part = blockIdx.x % PC;
  // x lines of plane z are the row groups z*NG .. z*NG + NG - 1 of pass 0 / 4; its y lines the
  // groups z*NG .. of pass 1 / 3 (outer index z). __syncthreads between groups: the next group
  // reuses S.
  if constexpr (DIR == 0) {
    for (int gg = part; gg < NG; gg += PC) { fft_lines<T, N1, N2, 0>(I, z * NG + gg, S); __syncthreads(); }
    cluster_sync_all();
    for (int gg = part; gg < NG; gg += PC) { fft_lines<T, N1, N2, 1>(I, z * NG + gg, S); __syncthreads(); }
  } else {
    for (int gg = part; gg < NG; gg += PC) { fft_lines<T, N1, N2, 3>(I, z * NG + gg, S); __syncthreads(); }
    cluster_sync_all();
    for (int gg = part; gg < NG; gg += PC) { fft_lines<T, N1, N2, 4>(I, z * NG + gg, S); __syncthreads(); }
  }
}

// The kernels: without a register hint, and (FP32 at N = 256, measured 2 droplets: 0.158 / 0.160
// ms per step against 0.160 / 0.166 ms without it) with 3 CTAs per SM; other sizes spill with it.
template <class T, int N1, int N2, int DIR>
__global__ void __cluster_dims__(plane_parts<N1 * N2>(), 1, 1) __launch_bounds__(lines_per_cta<N1 * N2>() * N2)
    k_fftr_plane(const InstDev<T>* __restrict__ insts) {
  plane_body<T, N1, N2, DIR>(insts);
}
template <class T, int N1, int N2, int DIR>
__global__ void __cluster_dims__(plane_parts<N1 * N2>(), 1, 1) __launch_bounds__(lines_per_cta<N1 * N2>() * N2, 3)
    k_fftr_plane3(const InstDev<T>* __restrict__ insts) {
  plane_body<T, N1, N2, DIR>(insts);
}
template <class T, int N1, int N2>
constexpr bool plane_hinted() { return sizeof(T) == 4 && N1 * N2 == 256; }

template <class T, int N1, int N2, int PASS>
void launch_pass(const Group<T>& g, cudaStream_t st) {
  constexpr int N = N1 * N2;
  constexpr int LB = lines_per_cta<N>();
  constexpr int axis = (PASS == 0 || PASS == 4) ? 0 : ((PASS == 1 || PASS == 3) ? 1 : 2);
  const int nblk = axis == 0 ? (N * N) / LB : N * (N / LB);
  k_fftr<T, N1, N2, PASS><<<dim3(nblk, g.n), LB * N2, smem_bytes<T, N1, N2>(axis), st>>>(g.d_inst);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) throw std::runtime_error(std::string("fft (register) launch: ") + cudaGetErrorString(e));
}

template <class T, int N1, int N2, int DIR>
void launch_plane(const Group<T>& g, cudaStream_t st) {
  constexpr int N = N1 * N2;
  constexpr int LB = lines_per_cta<N>();
  constexpr size_t smem = smem_bytes<T, N1, N2>(0) > smem_bytes<T, N1, N2>(1) ? smem_bytes<T, N1, N2>(0)
                                                                                : smem_bytes<T, N1, N2>(1);
  const dim3 grid(N * plane_parts<N>(), g.n);
  if constexpr (plane_hinted<T, N1, N2>()) k_fftr_plane3<T, N1, N2, DIR><<<grid, LB * N2, smem, st>>>(g.d_inst);
  else k_fftr_plane<T, N1, N2, DIR><<<grid, LB * N2, smem, st>>>(g.d_inst);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) throw std::runtime_error(std::string("fft (register, plane) launch: ") + cudaGetErrorString(e));
}

template <class T, int N1, int N2>
void prepare_size() {
  auto set = [](const void* f, size_t b) {
    cudaError_t e = cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)b);
    if (e != cudaSuccess) throw std::runtime_error(std::string("fft (register) smem attribute: ") + cudaGetErrorString(e));
  };
  set((const void*)k_fftr<T, N1, N2, 0>, smem_bytes<T, N1, N2>(0));
  set((const void*)k_fftr<T, N1, N2, 1>, smem_bytes<T, N1, N2>(1));
  set((const void*)k_fftr<T, N1, N2, 2>, smem_bytes<T, N1, N2>(2));
  set((const void*)k_fftr<T, N1, N2, 3>, smem_bytes<T, N1, N2>(1));
  set((const void*)k_fftr<T, N1, N2, 4>, smem_bytes<T, N1, N2>(0));
  const size_t sp = smem_bytes<T, N1, N2>(0) > smem_bytes<T, N1, N2>(1) ? smem_bytes<T, N1, N2>(0) : smem_bytes<T, N1, N2>(1);
  if constexpr (plane_hinted<T, N1, N2>()) {
    set((const void*)k_fftr_plane3<T, N1, N2, 0>, sp);
    set((const void*)k_fftr_plane3<T, N1, N2, 1>, sp);
  } else {
    set((const void*)k_fftr_plane<T, N1, N2, 0>, sp);
    set((const void*)k_fftr_plane<T, N1, N2, 1>, sp);
  }
}

template <class T, int N1, int N2>
void launch_size(const Group<T>& g, int pass, cudaStream_t st) {
  switch (pass) {
    case 0: launch_pass<T, N1, N2, 0>(g, st); break;
    case 1: launch_pass<T, N1, N2, 1>(g, st); break;
    case 2: launch_pass<T, N1, N2, 2>(g, st); break;
    case 3: launch_pass<T, N1, N2, 3>(g, st); break;
    default: launch_pass<T, N1, N2, 4>(g, st); break;
  }
}

// The sizes with a register kernel: N = N1*N2 with N2 a power of two dividing N1 and N2 as
// large as that allows up to sqrt(N). Others use the shared-memory Stockham kernels.
#define TTSH_FFTREG_SIZES(X) \
  X(8, 4, 2)                 \
  X(16, 4, 4)                \
  X(24, 12, 2)               \
  X(32, 8, 4)                \
  X(48, 12, 4)               \
  X(64, 8, 8)                \
  X(96, 24, 4)               \
  X(128, 16, 8)              \
  X(160, 40, 4)              \
  X(192, 24, 8)              \
  X(256, 16, 16)             \
  X(512, 32, 16)

template <class T>
bool reg_supported(int N) {
  switch (N) {
#define X(n, a, b) case n: return true;
    TTSH_FFTREG_SIZES(X)
#undef X
    default: return false;
  }
}

template <class T>
void reg_prepare(int N) {
  switch (N) {
#define X(n, a, b) case n: prepare_size<T, a, b>(); break;
    TTSH_FFTREG_SIZES(X)
#undef X
    default: break;
  }
}

template <class T>
bool reg_plane_launch(const Group<T>& g, int dir, cudaStream_t st) {
  switch (g.N) {
#define X(n, a, b) case n: if (dir == 0) launch_plane<T, a, b, 0>(g, st); else launch_plane<T, a, b, 1>(g, st); return true;
    TTSH_FFTREG_SIZES(X)
#undef X
    default: return false;
  }
}

template <class T>
bool reg_launch(const Group<T>& g, int pass, cudaStream_t st) {
  switch (g.N) {
#define X(n, a, b) case n: launch_size<T, a, b>(g, pass, st); return true;
    TTSH_FFTREG_SIZES(X)
#undef X
    default: return false;
  }
}

}  // namespace fftreg
}  // namespace ttsh
