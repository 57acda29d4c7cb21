// fftreg_impl.cuh — the register-resident FFT pass kernel and its size table, instantiated for
// one arithmetic type by fftreg_f32.cu / fftreg_f64.cu (two translation units build in parallel).
#pragma once
#include <cuda.h>
#include <cudaTypedefs.h>

#include <cmath>
#include <stdexcept>
#include <string>
#include <vector>

#include "common.cuh"
#include "fftreg.cuh"
#include "kernels.h"

namespace ttsh {
namespace fftreg {

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

// __constant__ copies of the per-size twiddle tables (exp(-2 pi i k / N), the values of the
// FP64-built table in global memory), filled by reg_twiddles when a size is prepared (every
// register FFT kernel of the size reads them).
#define X(n, a, b)                                                                     \
  __constant__ float2 c_twf_##n[n];                                                    \
  __constant__ double2 c_twd_##n[n];                                                   \
  template <>                                                                          \
  __device__ __forceinline__ float2 ctw<float2, n>(int k) { return c_twf_##n[k]; }      \
  template <>                                                                          \
  __device__ __forceinline__ double2 ctw<double2, n>(int k) { return c_twd_##n[k]; }
TTSH_FFTREG_SIZES(X)
#undef X

template <class T>
void reg_twiddles(int N) {
  typedef typename CxT<T>::type C;
  // exp(-2 pi i k / N) formed in FP64 and rounded to T, as the table in global memory is
  const double kPi = 3.1415926535897932384626433832795;
  std::vector<C> tw(N);
  for (int k = 0; k < N; ++k) {
    const double a = -2.0 * kPi * (double)k / (double)N;
    tw[k].x = (T)std::cos(a);
    tw[k].y = (T)std::sin(a);
  }
  cudaError_t e = cudaSuccess;
  switch (N) {
#define X(n, a, b)                                                                          \
  case n:                                                                                   \
    if constexpr (sizeof(T) == 4) e = cudaMemcpyToSymbol(c_twf_##n, tw.data(), n * sizeof(C)); \
    else e = cudaMemcpyToSymbol(c_twd_##n, tw.data(), n * sizeof(C));                       \
    break;
    TTSH_FFTREG_SIZES(X)
#undef X
    default: break;
  }
  if (e != cudaSuccess) throw std::runtime_error(std::string("fft (register) twiddle table: ") + cudaGetErrorString(e));
}


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

struct NoOp {
  __device__ __forceinline__ void operator()() const {}
};

// The four-step twiddle w_N^k of a line group from the __constant__ table (CONST) or the table in
// global memory. A warp's loads of the constant table are served one distinct address at a time:
// for y and z lines the index takes two values per warp; for x lines it takes N2 (the thread's
// column index), and the constant table is faster only up to N2 = 8 (measured: x+y and y+x per
// plane -8 % at 128^3, N2 = 8; +25 % at 256^3, N2 = 16).
template <class C, bool INV, int N, bool CONST>
__device__ __forceinline__ C tw4(const C* tab, int k) {
  if constexpr (CONST) {
    C w = ctw<C, N>(k);
    if (INV) w.y = -w.y;
    return w;
  } else {
    return tw<C, INV>(tab, k);
  }
}

// PASS: 0 forward x, 1 forward y, 2 forward z + Poisson multiplier + inverse z, 3 inverse y,
// 4 inverse x scaled by 1/N^3. One call transforms line group g of the pass (LB lines) with the
// CTA's threads; S is the CTA's shared memory. SIN (z pass only): the group's input is already in
// shared memory, In[z * LB + line]; `after` runs once every thread has read it (In may then be
// refilled).
template <class T, int N1, int N2, int PASS, bool SIN = false, class F = NoOp>
__device__ __forceinline__ void fft_lines(const InstDev<T>& I, int g, typename CxT<T>::type* S,
                                          const typename CxT<T>::type* In = nullptr, F after = F()) {
  typedef typename CxT<T>::type C;
  constexpr int N = N1 * N2;
  constexpr int LB = lines_per_cta<N>();
  constexpr int OW = N1 / N2;  // k1 rows owned by each thread in the second step
  constexpr int axis = (PASS == 0 || PASS == 4) ? 0 : ((PASS == 1 || PASS == 3) ? 1 : 2);
  constexpr bool TW4C = axis != 0 || N2 <= 8;  // four-step twiddles from the constant table
  static_assert(!SIN || axis == 2, "shared-memory input: z pass only");
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
    if constexpr (SIN) {
#pragma unroll
      for (int n1 = 0; n1 < N1; ++n1) v[n1] = In[(N2 * n1 + j) * LB + l];
    } else {
#pragma unroll
      for (int n1 = 0; n1 < N1; ++n1) v[n1] = W[base + (size_t)(N2 * n1 + j) * stride];
    }
    if constexpr (PASS == 0 && sizeof(T) == 4) {
      // FP32: both parts of the packed source brought to the same size (pow2_norm, common.cuh)
      if (I.wmax) {
        const T su = pow2_norm(I.wmax[0]), sp = pow2_norm(I.wmax[1]);
#pragma unroll
        for (int n1 = 0; n1 < N1; ++n1) { v[n1].x *= su; v[n1].y *= sp; }
      }
    }
    Dft<C, N1, false, N>::run(v, tab, N2);
#pragma unroll
    for (int k1 = 0; k1 < N1; ++k1) S[sidx(k1, j)] = (k1 > 0 && j > 0) ? cmul(v[k1], tw4<C, false, N, TW4C>(tab, j * k1)) : v[k1];
    __syncthreads();
    after();
#pragma unroll
    for (int o = 0; o < OW; ++o) {
      const int k1 = j + N2 * o;
      C u[N2];
#pragma unroll
      for (int n2 = 0; n2 < N2; ++n2) u[n2] = S[sidx(k1, n2)];
      Dft<C, N2, false, N>::run(u, tab, N1);
      if constexpr (PASS == 2) {
        // spectrum element z = k1 + N1*k2 of the line (x = xl, y = yl): multiply, go back
#pragma unroll
        for (int k2 = 0; k2 < N2; ++k2) u[k2] = poisson_mul(u[k2], I, xl, yl, k1 + N1 * k2);
        Dft<C, N2, true, N>::run(u, tab, N1);
#pragma unroll
        for (int n2 = 0; n2 < N2; ++n2) S[sidx(k1, n2)] = (n2 > 0 && k1 > 0) ? cmul(u[n2], tw4<C, true, N, TW4C>(tab, n2 * k1)) : u[n2];
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
      Dft<C, N1, true, N>::run(x, tab, N2);
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
      Dft<C, N2, true, N>::run(u, tab, N1);
#pragma unroll
      for (int n2 = 0; n2 < N2; ++n2) S[sidx(k1, n2)] = (n2 > 0 && k1 > 0) ? cmul(u[n2], tw4<C, true, N, TW4C>(tab, n2 * k1)) : u[n2];
    }
    __syncthreads();
    C x[N1];
#pragma unroll
    for (int k1 = 0; k1 < N1; ++k1) x[k1] = S[sidx(k1, j)];
    Dft<C, N1, true, N>::run(x, tab, N2);
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

// ---- the z pass with its input staged by the tensor memory accelerator (FP32) ----
// Persistent CTAs: CTA b takes the z-line groups b, b + grid, ... of every droplet of the size
// group. A group's input, the LB x 1 x N box (x, y, z) of the droplet's complex field, is copied
// into one of ZST shared-memory stages by cp.async.bulk.tensor (one instruction per 256 z-planes),
// ZST groups ahead of the one being transformed; an mbarrier per stage counts the bytes in.
// Arithmetic and output are those of k_fftr<float, N1, N2, 2>.
constexpr int ZST = 2;

__device__ __forceinline__ unsigned smem_u32(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void mbar_init(uint64_t* b, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(smem_u32(b)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_fence_init() { asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory"); }
__device__ __forceinline__ void mbar_expect_tx(uint64_t* b, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(smem_u32(b)), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* b, unsigned parity) {
  unsigned done;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(done)
      : "r"(smem_u32(b)), "r"(parity)
      : "memory");
  return done != 0;
}
// Waits for phase `parity` of the barrier for at most `limit` SM clocks (2^31, about a second, on
// the step); false when that limit ran out.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* b, unsigned parity, long long limit = 1ll << 31) {
  if (mbar_try_wait(b, parity)) return true;
  const long long t0 = clock64();
  while (!mbar_try_wait(b, parity))
    if (clock64() - t0 > limit) return false;
  return true;
}
__device__ __forceinline__ void tma_load_3d(void* dst, const CUtensorMap* map, int x, int y, int z, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];\n" ::"r"(
          smem_u32(dst)),
      "l"(map), "r"(x), "r"(y), "r"(z), "r"(smem_u32(bar))
      : "memory");
}

template <int N>
constexpr size_t zt_smem() {
  return (size_t)(ZST + 1) * N * lines_per_cta<N>() * sizeof(float2) + ZST * sizeof(uint64_t);
}
template <int N>
constexpr int zt_min_blocks() { return 2 * zt_smem<N>() <= 227 * 1024 ? 2 : 1; }
// The sizes with the staged z pass (on request, TTSH_ZTMA=1): CTAs of 256 threads, two per SM
// (N = 256). The directly loading kernel is faster and is the default, per step (ms, CUDA
// events): 64 x 128^3 0.573 against 0.644 staged (128-thread CTAs: a quarter of the direct
// kernel's resident warps); 512^3 0.84 against 0.98 (240 registers a thread, one CTA per SM);
// 2 x 256^3 0.128 against 0.152 once the twiddles come from the constant table.
template <int N1, int N2>
constexpr bool zt_has() {
  return lines_per_cta<N1 * N2>() == 16 && lines_per_cta<N1 * N2>() * N2 == 256 && N1 * N2 <= 256 &&
         zt_min_blocks<N1 * N2>() == 2;
}

template <int N1, int N2>
__global__ void __launch_bounds__(lines_per_cta<N1 * N2>() * N2, zt_min_blocks<N1 * N2>())
    k_fftz_tma(const InstDev<float>* __restrict__ insts, const CUtensorMap* __restrict__ maps, int ninst,
               int* __restrict__ err, int drop_first) {
  typedef float2 C;
  constexpr int N = N1 * N2, LB = lines_per_cta<N>(), NGX = N / LB, NG = N * NGX;
  constexpr int NBOX = (N + 255) / 256, BZ = N / NBOX;
  static_assert(NBOX * BZ == N, "the boxes tile a line");
  constexpr unsigned STAGE = (unsigned)(N * LB * sizeof(C));
  extern __shared__ __align__(1024) unsigned char zt_smem_raw[];  // TMA boxes want a 128-byte aligned base
  C* In = reinterpret_cast<C*>(zt_smem_raw);                // [ZST][N][LB]: the box layout
  C* S = In + (size_t)ZST * N * LB;                          // the transposes, N * LB
  uint64_t* bar = reinterpret_cast<uint64_t*>(S + (size_t)N * LB);  // [ZST]
  const int total = ninst * NG, tid = threadIdx.x;
  auto issue = [&](int g, int s) {
    const int inst = g / NG, gl = g - inst * NG;
    const int y = gl / NGX, x = (gl - y * NGX) * LB;
    mbar_expect_tx(&bar[s], STAGE);
#pragma unroll
    for (int b = 0; b < NBOX; ++b)
      tma_load_3d(In + ((size_t)s * N + (size_t)b * BZ) * LB, maps + inst, 2 * x, y, b * BZ, &bar[s]);
  };
  // issued[s] (used by thread 0): the CTA-local index k of the last group whose copy went to stage
  // s, or -1
  int issued[ZST];
#pragma unroll
  for (int s = 0; s < ZST; ++s) issued[s] = -1;
  if (tid == 0) {
    for (int s = 0; s < ZST; ++s) mbar_init(&bar[s], 1);
    mbar_fence_init();
  }
  __syncthreads();
  if (tid == 0)
    for (int s = 0; s < ZST; ++s)
      if (blockIdx.x + s * gridDim.x < total && !(drop_first && s == 0)) {
        issue(blockIdx.x + s * gridDim.x, s);
        issued[s] = s;
      }
  // the failure test shortens the wait so that the dropped copy's wait runs out quickly
  const long long limit = drop_first ? (1ll << 20) : (1ll << 31);
  int k = 0;
  bool ok = true;
  for (int g = blockIdx.x; g < total; g += gridDim.x, ++k) {
    const int s = k % ZST;
    // every thread observes the copy complete (acquire); the CTA goes on only if all did
    ok = __syncthreads_and(mbar_wait_bounded(&bar[s], (unsigned)(k / ZST) & 1u, limit)) != 0;
    if (!ok) break;
    const int inst = g / NG, gn = g + ZST * gridDim.x;
    fft_lines<float, N1, N2, 2, true>(insts[inst], g - inst * NG, S, In + (size_t)s * N * LB, [&] {
      if (tid == 0 && gn < total) {
        issue(gn, s);
        issued[s] = k + ZST;
      }
    });
  }
  if (!ok) {
    // a copy did not complete in time: report it, then wait for this CTA's copies still in
    // flight (issued to a stage for group k or later) before its shared memory is released.
    // That wait is bounded too (2^31 clocks); were it to run out, the CTA would leave with a copy
    // still writing, and the context as a whole is to be treated as unreliable after this error.
    if (tid == 0) {
      atomicExch(err, 1);
      for (int q = 0; q < ZST; ++q)
        if (issued[q] >= k) mbar_wait_bounded(&bar[q], (unsigned)(issued[q] / ZST) & 1u);
    }
    __syncthreads();
  }
}

template <int N1, int N2>
void launch_zt(const Group<float>& g, cudaStream_t st) {
  constexpr int N = N1 * N2, LB = lines_per_cta<N>();
  const int total = g.n * N * (N / LB);
  const int grid = total < g.zt_grid ? total : g.zt_grid;
  k_fftz_tma<N1, N2><<<grid, LB * N2, zt_smem<N>(), st>>>(g.d_inst, reinterpret_cast<const CUtensorMap*>(g.d_tmz),
                                                          g.n, g.d_err, g.zt_drop);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) throw std::runtime_error(std::string("fft (staged z) launch: ") + cudaGetErrorString(e));
}

// CTAs of the staged z pass that fit on the device at once (0: the size has none).
template <int N1, int N2>
int zt_prepare() {
  if constexpr (!zt_has<N1, N2>()) {
    return 0;
  } else {
    constexpr int N = N1 * N2, LB = lines_per_cta<N>();
    cudaError_t e = cudaFuncSetAttribute((const void*)k_fftz_tma<N1, N2>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)zt_smem<N>());
    if (e != cudaSuccess) throw std::runtime_error(std::string("fft (staged z) smem attribute: ") + cudaGetErrorString(e));
    int dev = 0, sms = 0, per = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_fftz_tma<N1, N2>, LB * N2, zt_smem<N>());
    if (e != cudaSuccess) throw std::runtime_error(std::string("fft (staged z) occupancy: ") + cudaGetErrorString(e));
    return sms * per;
  }
}

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
    case 2:
      if constexpr (sizeof(T) == 4 && zt_has<N1, N2>()) {
        if (g.zt_grid > 0 && g.d_tmz) {
          launch_zt<N1, N2>(g, st);
          break;
        }
      }
      launch_pass<T, N1, N2, 2>(g, st);
      break;
    case 3: launch_pass<T, N1, N2, 3>(g, st); break;
    default: launch_pass<T, N1, N2, 4>(g, st); break;
  }
}

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

// The descriptor of one droplet's complex field for the staged z pass: 3-D, x in FP32 words
// (2N, re/im interleaved), y, z; the box is LB lines x 1 row x N / NBOX planes.
template <int N1, int N2>
void zt_encode(const void* W, CUtensorMap* map) {
  if constexpr (zt_has<N1, N2>()) {
    constexpr int N = N1 * N2, LB = lines_per_cta<N>(), NBOX = (N + 255) / 256;
    static PFN_cuTensorMapEncodeTiled_v12000 encode = nullptr;
    if (!encode) {
      void* fn = nullptr;
      cudaDriverEntryPointQueryResult q{};
      if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) != cudaSuccess ||
          q != cudaDriverEntryPointSuccess || !fn)
        throw std::runtime_error("cuTensorMapEncodeTiled is not available from the driver");
      encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
    }
    const cuuint64_t dims[3] = {2ull * N, (cuuint64_t)N, (cuuint64_t)N};
    const cuuint64_t strides[2] = {2ull * N * sizeof(float), 2ull * N * N * sizeof(float)};
    const cuuint32_t box[3] = {2u * LB, 1u, (cuuint32_t)(N / NBOX)};
    const cuuint32_t es[3] = {1u, 1u, 1u};
    const CUresult r = encode(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, const_cast<void*>(W), dims, strides, box, es,
                              CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                              CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) throw std::runtime_error("cuTensorMapEncodeTiled failed (" + std::to_string((int)r) + ")");
  }
}

inline void reg_zt_encode(int N, const void* W, CUtensorMap* map) {
  switch (N) {
#define X(n, a, b) case n: zt_encode<a, b>(W, map); break;
    TTSH_FFTREG_SIZES(X)
#undef X
    default: break;
  }
}

inline int reg_zt_prepare(int N) {
  switch (N) {
#define X(n, a, b) case n: return zt_prepare<a, b>();
    TTSH_FFTREG_SIZES(X)
#undef X
    default: return 0;
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
