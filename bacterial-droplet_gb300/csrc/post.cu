// post.cu — readDraw.py's per-snapshot reductions on the device: the phi-weighted centroid
// (calculate_centroid, readDraw.py:30-52), the z-slice through it (readDraw.py:222-233) and the
// 2D vorticities of (vx, vy) and (px, py) on that slice (readDraw.py:236-237) with op.py's
// 4th-order periodic first derivatives (d1xO4 / d1yO4, op.py:3-13).
//
// readDraw indexes the reshaped field as field[i][j][k] = (y, x, z), so its "centroid_x" is the
// mean y, "centroid_y" the mean x and "centroid_z" the mean z; the slice field[:, :, idx3] is the
// [y][x] plane at z = idx3. The outputs here keep that order.
#include <cmath>
#include <stdexcept>

#include "common.cuh"
#include "kernels.h"

namespace ttsh {

namespace {

constexpr int CB = 256, CT = 256;

// Per-block FP64 partial sums of phi, phi*y, phi*x, phi*z (fixed reduction order).
template <class T>
__global__ void __launch_bounds__(CT) k_centroid(const InstDev<T>* __restrict__ insts, int inst, int par,
                                                 double* __restrict__ part) {
  const InstDev<T>& I = insts[inst];
  const int N = I.N;
  const long n = (long)N * N * N;
  const T* phi = I.phi[par];
  double s[4] = {0, 0, 0, 0};
  for (long i = (long)blockIdx.x * CT + threadIdx.x; i < n; i += (long)CB * CT) {
    const double f = (double)phi[i] + (I.phic ? (double)I.phic[i] : 0.0);  // compensated in the fused form
    const int x = (int)(i % N), y = (int)((i / N) % N), z = (int)(i / ((long)N * N));
    s[0] += f;
    s[1] += f * y;
    s[2] += f * x;
    s[3] += f * z;
  }
  __shared__ double sh[4][CT / 32];
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    for (int o = 16; o > 0; o >>= 1) s[q] += __shfl_down_sync(0xffffffffu, s[q], o);
    if ((threadIdx.x & 31) == 0) sh[q][threadIdx.x >> 5] = s[q];
  }
  __syncthreads();
  if (threadIdx.x < 4) {
    double a = 0;
    for (int w = 0; w < CT / 32; ++w) a += sh[threadIdx.x][w];
    part[blockIdx.x * 4 + threadIdx.x] = a;
  }
}

// The z = zs plane of the 7 snapshot fields, [y][x], and the two vorticities.
template <class T>
__global__ void k_slice(const InstDev<T>* __restrict__ insts, int inst, int par, int zs, double* __restrict__ out) {
  const InstDev<T>& I = insts[inst];
  const int N = I.N;
  const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y;
  if (x >= N) return;
  const size_t NN = (size_t)N * N, plane = (size_t)zs * NN;
  const size_t o = (size_t)y * N + x;
  // field q (vx vy vz px py pz phi) at flat index i: in the fused form the compensated value
  auto val = [&](int q, size_t i) -> double {
    if (q == 6) return (double)I.phi[par][i] + (I.phic ? (double)I.phic[i] : 0.0);
    const T* f = q < 3 ? I.U[q] : I.P[q - 3];
    double v = (double)f[i];
    if (q < 3 && I.lo[q]) v += (double)__bfloat162float(I.lo[q][i]);
    return v;
  };
#pragma unroll
  for (int q = 0; q < 7; ++q) out[q * NN + o] = val(q, plane + o);
  // op.py: d1xO4(u) = (u[x-2] - 8u[x-1] + 8u[x+1] - u[x+2]) / (12h) along x, d1yO4 along y
  const double c = 1.0 / (12 * (double)I.ph.h);
  auto at = [&](int q, int yy, int xx) {
    yy = (yy % N + N) % N;
    xx = (xx % N + N) % N;
    return val(q, plane + (size_t)yy * N + xx);
  };
  auto dx = [&](int q) {
    return c * (at(q, y, x - 2) - 8 * at(q, y, x - 1) + 8 * at(q, y, x + 1) - at(q, y, x + 2));
  };
  auto dy = [&](int q) {
    return c * (at(q, y - 2, x) - 8 * at(q, y - 1, x) + 8 * at(q, y + 1, x) - at(q, y + 2, x));
  };
  out[7 * NN + o] = dx(1) - dy(0);  // vortex = d1xO4(vy) - d1yO4(vx)  (readDraw.py:236)
  out[8 * NN + o] = dx(4) - dy(3);  // Pvortex = d1xO4(py) - d1yO4(px) (readDraw.py:237)
}

// FP64 <-> FP32 conversion of one field on the device, for the host interface of the FP32 forms:
// the caller's FP64 arrays are read (or written) as they are, in device memory or straight in
// host memory the device can address, and converted here (round to nearest), instead of element
// by element on the host. k_to_f64 multiplies by the power of two whose float bits *scale_bits
// record (pow2_denorm; nullptr: 1), read on the device so that no host wait is needed for it.
__global__ void k_to_f32(const double* __restrict__ src, float* __restrict__ dst, size_t n) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    dst[i] = __double2float_rn(src[i]);
}
__global__ void k_to_f64(const float* __restrict__ src, size_t stride, double* __restrict__ dst, size_t n,
                         const int* __restrict__ scale_bits) {
  const double scale = scale_bits ? (double)pow2_denorm(*scale_bits) : 1.0;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    dst[i] = (double)src[i * stride] * scale;
}
// a strided FP64 field (p_v or p_p of the packed complex W) into a contiguous one
__global__ void k_gather_f64(const double* __restrict__ src, size_t stride, double* __restrict__ dst, size_t n) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    dst[i] = src[i * stride];
}

// The compensated fields of the fused FP32 form: hi = the FP64 value rounded to FP32 and the
// remainder in bf16 (lo) or, for phi, in FP32 (lo32, its update's compensation field).
// hi and lo are read / written with `stride` (2: one half of an interleaved pair field).
__global__ void k_split(const double* __restrict__ src, float* __restrict__ hi, __nv_bfloat16* __restrict__ lo,
                        float* __restrict__ lo32, size_t n, int stride) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const double v = src[i];
    const float h = __double2float_rn(v);
    hi[stride * i] = h;
    const double r = v - (double)h;  // exact
    if (lo) lo[stride * i] = __double2bfloat16(r);
    if (lo32) lo32[i] = __double2float_rn(r);
  }
}
__global__ void k_join(const float* __restrict__ hi, const __nv_bfloat16* __restrict__ lo, const float* __restrict__ lo32,
                       double* __restrict__ dst, size_t n, int stride) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    double v = (double)hi[stride * i];
    if (lo) v += (double)__bfloat162float(lo[stride * i]);
    if (lo32) v += (double)lo32[i];
    dst[i] = v;
  }
}

inline void check_conv(const char* what) {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) throw std::runtime_error(std::string(what) + " launch: " + cudaGetErrorString(e));
}

}  // namespace

void launch_split(const double* src, float* hi, __nv_bfloat16* lo, float* lo32, size_t n, int stride, cudaStream_t st) {
  k_split<<<1216, 256, 0, st>>>(src, hi, lo, lo32, n, stride);
  check_conv("split");
}
void launch_join(const float* hi, const __nv_bfloat16* lo, const float* lo32, double* dst, size_t n, int stride,
                 cudaStream_t st) {
  k_join<<<1216, 256, 0, st>>>(hi, lo, lo32, dst, n, stride);
  check_conv("join");
}

void launch_to_f32(const double* src, float* dst, size_t n, cudaStream_t st) {
  k_to_f32<<<1216, 256, 0, st>>>(src, dst, n);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) throw std::runtime_error(std::string("conversion launch: ") + cudaGetErrorString(e));
}
void launch_to_f64(const float* src, size_t stride, double* dst, size_t n, const int* scale_bits, cudaStream_t st) {
  k_to_f64<<<1216, 256, 0, st>>>(src, stride, dst, n, scale_bits);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) throw std::runtime_error(std::string("conversion launch: ") + cudaGetErrorString(e));
}
void launch_gather_f64(const double* src, size_t stride, double* dst, size_t n, cudaStream_t st) {
  k_gather_f64<<<1216, 256, 0, st>>>(src, stride, dst, n);
  check_conv("gather");
}

int centroid_blocks() { return CB; }

template <class T>
void launch_centroid(const InstDev<T>* d_all, int inst, int par, double* part, cudaStream_t st) {
  k_centroid<T><<<CB, CT, 0, st>>>(d_all, inst, par, part);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) throw std::runtime_error(std::string("centroid launch: ") + cudaGetErrorString(e));
}

template <class T>
void launch_slice(const InstDev<T>* d_all, int inst, int par, int N, int zs, double* out, cudaStream_t st) {
  k_slice<T><<<dim3((N + 127) / 128, N), 128, 0, st>>>(d_all, inst, par, zs, out);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) throw std::runtime_error(std::string("slice launch: ") + cudaGetErrorString(e));
}

template void launch_centroid<float>(const InstDev<float>*, int, int, double*, cudaStream_t);
template void launch_centroid<double>(const InstDev<double>*, int, int, double*, cudaStream_t);
template void launch_slice<float>(const InstDev<float>*, int, int, int, int, double*, cudaStream_t);
template void launch_slice<double>(const InstDev<double>*, int, int, int, int, double*, cudaStream_t);

}  // namespace ttsh
