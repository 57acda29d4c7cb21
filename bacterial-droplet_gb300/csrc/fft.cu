// fft.cu — hand-written batched 3D FFT Poisson solve (replaces the reference's
// cufftExecZ2Z forward/inverse pair and getStream modes 1 and 2, TTSH3D.cu:635-691).
//
// Both projections of a step are solved with ONE complex transform: the packed
// field W = div(u*)/dt + i div(P*)/dt is transformed, multiplied by the real, even
// multiplier -1/k^2, and transformed back, so Re W = p_v and Im W = p_p (the
// multiplier keeps the Hermitian symmetry of each real part separately).
//
// Each pass moves LB lines of length N through shared memory and runs a
// mixed-radix Stockham autosort FFT there (radix 4, 2, 3, 5; natural order in and
// out; the formulation of Govindaraju et al., SC'08). Passes:
//   0 forward x   1 forward y   2 forward z -> divide -> inverse z
//   3 inverse y   4 inverse x, scaled by 1/N^3 (getStream mode 2, :684-690)
// Twiddles come from a table exp(-2 pi i k/N) built on the host in FP64.
#include <cstdio>
#include <stdexcept>

#include "common.cuh"
#include "fftreg.cuh"
#include "kernels.h"

namespace ttsh {

using fftreg::poisson_mul;
using fftreg::scale_n3;

namespace {

constexpr int FFT_THREADS = 256;

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

// Twiddle exp(sign * 2 pi i k / N) with sign -1 (forward) or +1 (inverse).
template <class C>
__device__ __forceinline__ C twid(const C* tw, int k, bool inv) {
  C t = __ldg(tw + k);
  if (inv) t.y = -t.y;
  return t;
}

// One Stockham stage of radix R on LB lines of pitch `pitch`.
template <class C, int R>
__device__ __forceinline__ void stage(const C* __restrict__ src, C* __restrict__ dst, int N, int LB, int pitch, int Ns,
                                      const C* tw, bool inv) {
  const int M = N / R;
  const int tstride = N / (Ns * R);
  for (int b = threadIdx.x; b < LB * M; b += blockDim.x) {
    const int l = b / M, j = b - l * M;
    const int k = j % Ns;
    const C* s = src + l * pitch;
    C v[R];
#pragma unroll
    for (int r = 0; r < R; ++r) {
      v[r] = s[j + r * M];
      if (r > 0 && k > 0) v[r] = cmul(v[r], twid(tw, r * k * tstride, inv));
    }
    C o[R];
    if (R == 2) {
      o[0] = cadd(v[0], v[1]);
      o[1] = csub(v[0], v[1]);
    } else if (R == 4) {
      C a = cadd(v[0], v[2]), b2 = csub(v[0], v[2]), c = cadd(v[1], v[3]), d = csub(v[1], v[3]);
      // multiply d by -i (forward) or +i (inverse)
      C dd;
      if (inv) { dd.x = -d.y; dd.y = d.x; } else { dd.x = d.y; dd.y = -d.x; }
      o[0] = cadd(a, c);
      o[2] = csub(a, c);
      o[1] = cadd(b2, dd);
      o[3] = csub(b2, dd);
    } else {
      // small DFT from the same table: w_R^(q r) = w_N^((q r mod R) N/R)
#pragma unroll
      for (int q = 0; q < R; ++q) {
        C acc = v[0];
#pragma unroll
        for (int r = 1; r < R; ++r) acc = cadd(acc, cmul(v[r], twid(tw, ((q * r) % R) * M, inv)));
        o[q] = acc;
      }
    }
    C* d = dst + l * pitch + (j / Ns) * Ns * R + k;
#pragma unroll
    for (int r = 0; r < R; ++r) d[r * Ns] = o[r];
  }
}

// Runs all stages; returns the buffer holding the result.
template <class C>
__device__ C* run_fft(C* a, C* b, int N, int LB, int pitch, const int* radix, int nst, const C* tw, bool inv) {
  int Ns = 1;
  for (int s = 0; s < nst; ++s) {
    const int R = radix[s];
    if (R == 4) stage<C, 4>(a, b, N, LB, pitch, Ns, tw, inv);
    else if (R == 2) stage<C, 2>(a, b, N, LB, pitch, Ns, tw, inv);
    else if (R == 3) stage<C, 3>(a, b, N, LB, pitch, Ns, tw, inv);
    else stage<C, 5>(a, b, N, LB, pitch, Ns, tw, inv);
    __syncthreads();
    C* t = a; a = b; b = t;
    Ns *= R;
  }
  return a;
}

template <class T, int PASS>
__global__ void __launch_bounds__(FFT_THREADS) k_fft(const InstDev<T>* __restrict__ insts, int LB) {
  typedef typename CxT<T>::type C;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const InstDev<T>& I = insts[blockIdx.y];
  const int N = I.N;
  const int pitch = N + 1;
  C* buf0 = reinterpret_cast<C*>(smem_raw);
  C* buf1 = buf0 + LB * pitch;
  C* W = I.W;
  const int axis = (PASS == 0 || PASS == 4) ? 0 : ((PASS == 1 || PASS == 3) ? 1 : 2);
  const size_t NN = (size_t)N * N;
  const int g = blockIdx.x;
  size_t base0 = 0, stride = 1;
  int lineY = 0, x0 = 0;
  if (axis == 0) {
    base0 = (size_t)g * LB * N;
  } else {
    const int ng = N / LB;
    const int outer = g / ng;
    x0 = (g - outer * ng) * LB;
    if (axis == 1) { base0 = (size_t)outer * NN + x0; stride = N; }
    else { base0 = (size_t)outer * N + x0; stride = NN; lineY = outer; }
  }
  // load (FP32, first forward pass: both parts of the packed source brought to the same size,
  // pow2_norm in common.cuh)
  T su = T(1), sp = T(1);
  if constexpr (PASS == 0 && sizeof(T) == 4) {
    if (I.wmax) {
      su = pow2_norm(I.wmax[0]);
      sp = pow2_norm(I.wmax[1]);
    }
  }
  for (int t = threadIdx.x; t < LB * N; t += blockDim.x) {
    int l, e;
    size_t src;
    if (axis == 0) { l = t / N; e = t - l * N; src = base0 + t; }
    else { e = t / LB; l = t - e * LB; src = base0 + (size_t)e * stride + l; }
    C v = W[src];
    if constexpr (PASS == 0 && sizeof(T) == 4) { v.x *= su; v.y *= sp; }
    buf0[l * pitch + e] = v;
  }
  __syncthreads();
  const bool inv = (PASS == 3 || PASS == 4);
  C* res = run_fft<C>(buf0, buf1, N, LB, pitch, I.radix, I.nstages, I.tw, inv);
  if (PASS == 2) {
    for (int t = threadIdx.x; t < LB * N; t += blockDim.x) {
      const int l = t / N, e = t - l * N;
      res[l * pitch + e] = poisson_mul(res[l * pitch + e], I, x0 + l, lineY, e);
    }
    __syncthreads();
    C* other = (res == buf0) ? buf1 : buf0;
    res = run_fft<C>(res, other, N, LB, pitch, I.radix, I.nstages, I.tw, true);
  }
  // store
  for (int t = threadIdx.x; t < LB * N; t += blockDim.x) {
    int l, e;
    size_t dst;
    if (axis == 0) { l = t / N; e = t - l * N; dst = base0 + t; }
    else { e = t / LB; l = t - e * LB; dst = base0 + (size_t)e * stride + l; }
    C v = res[l * pitch + e];
    if (PASS == 4) v = scale_n3(v, I);
    W[dst] = v;
  }
}

int pick_lb(int N, size_t csize) {
  int lb = 16;
  while (lb > 1 && (N % lb != 0 || 2 * (size_t)lb * (N + 1) * csize > 200 * 1024)) lb >>= 1;
  return lb;
}

template <class T, int PASS>
void launch_one(const Group<T>& g, cudaStream_t st) {
  typedef typename CxT<T>::type C;
  const int N = g.N;
  const int LB = fft_lines(g);
  const size_t smem = 2 * (size_t)LB * (N + 1) * sizeof(C);
  const int axis = (PASS == 0 || PASS == 4) ? 0 : ((PASS == 1 || PASS == 3) ? 1 : 2);
  const int nblk = axis == 0 ? (N * N) / LB : N * (N / LB);
  k_fft<T, PASS><<<dim3(nblk, g.n), FFT_THREADS, smem, st>>>(g.d_inst, LB);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) throw std::runtime_error(std::string("fft launch: ") + cudaGetErrorString(e));
}

}  // namespace

// One kernel serves every size, so its shared-memory limit is only ever raised: a group of one
// size must not lower the limit another size's launches need.
template <class T, int PASS>
void set_attr(int N) {
  typedef typename CxT<T>::type C;
  const size_t smem = 2 * (size_t)pick_lb(N, sizeof(C)) * (N + 1) * sizeof(C);
  cudaFuncAttributes fa{};
  cudaError_t e = cudaFuncGetAttributes(&fa, k_fft<T, PASS>);
  if (e == cudaSuccess && (size_t)fa.maxDynamicSharedSizeBytes >= smem) return;
  e = cudaFuncSetAttribute(k_fft<T, PASS>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) throw std::runtime_error(std::string("fft smem attribute: ") + cudaGetErrorString(e));
}

template <class T>
void fft_prepare(int N) {
  fftreg_prepare<T>(N);
  set_attr<T, 0>(N);
  set_attr<T, 1>(N);
  set_attr<T, 2>(N);
  set_attr<T, 3>(N);
  set_attr<T, 4>(N);
}

template <class T>
std::vector<int> fft_lb_candidates(int N) {
  typedef typename CxT<T>::type C;
  std::vector<int> r;
  for (int lb = pick_lb(N, sizeof(C)); lb >= 1; lb >>= 1)
    if (N % lb == 0) r.push_back(lb);
  return r;
}

template <class T>
int fft_lines(const Group<T>& g) {
  typedef typename CxT<T>::type C;
  const int mx = pick_lb(g.N, sizeof(C));  // the shared-memory limit is set for this one
  if (g.fft_lb == 0) return mx;
  if (g.fft_lb < 1 || g.fft_lb > mx || g.N % g.fft_lb != 0) throw std::runtime_error("fft: bad lines per CTA");
  return g.fft_lb;
}

template <class T>
size_t fft_smem_bytes(int N, int) {
  typedef typename CxT<T>::type C;
  return 2 * (size_t)pick_lb(N, sizeof(C)) * (N + 1) * sizeof(C);
}

template <class T>
void launch_fft_pass(const Group<T>& g, int pass, cudaStream_t st) {
  if (fftreg_launch<T>(g, pass, st)) return;
  switch (pass) {
    case 0: launch_one<T, 0>(g, st); break;
    case 1: launch_one<T, 1>(g, st); break;
    case 2: launch_one<T, 2>(g, st); break;
    case 3: launch_one<T, 3>(g, st); break;
    case 4: launch_one<T, 4>(g, st); break;
    default: throw std::runtime_error("bad fft pass");
  }
}

template std::vector<int> fft_lb_candidates<float>(int);
template std::vector<int> fft_lb_candidates<double>(int);
template int fft_lines<float>(const Group<float>&);
template int fft_lines<double>(const Group<double>&);
template void launch_fft_pass<float>(const Group<float>&, int, cudaStream_t);
template void launch_fft_pass<double>(const Group<double>&, int, cudaStream_t);
template size_t fft_smem_bytes<float>(int, int);
template void fft_prepare<float>(int);
template void fft_prepare<double>(int);
template size_t fft_smem_bytes<double>(int, int);

}  // namespace ttsh
