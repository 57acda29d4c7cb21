// kernels.h — host-side launch interface of libttsh's CUDA kernels (no device code here).
#pragma once
#include <cuda_runtime.h>

#include <vector>

namespace ttsh {

template <class T> struct InstDev;

// One group = instances of equal N sharing a device array of descriptors.
template <class T>
struct Group {
  InstDev<T>* d_inst;  // device array [n]
  int n;               // instances in the group
  int N;
  int fft_kind = 0;    // register-resident FFT kernels where the size has them: 0 one launch per
                       // axis pass, 2 x and y of a plane in one launch; 1: Stockham only
  int fft_lb = 0;      // Stockham lines per CTA (0: the largest power of two that fits)
  int zc[3] = {0, 64, 64};   // z-planes per CTA of fused_rhs, fused_div, fused_correct; 0: the
                             // persistent grid (equal shares of the group's sites per CTA)
  double tuned_ms[4] = {0, 0, 0, 0};  // the tuner's timings of this configuration (host record)
  double* red = nullptr;  // FP64 diagnostics partials of the whole group (n x 4 x blocks), contiguous
  // FP32 z pass staged by the tensor memory accelerator: a 3-D descriptor of each droplet's
  // complex field (device array of n CUtensorMap) and the persistent grid (0: not used)
  void* d_tmz = nullptr;
  int zt_grid = 0;
  int zt_drop = 0;       // failure test only (TTSH_TEST_DROP_STAGED_COPY=1): each CTA of the staged
                         // z pass skips its first copy, so that its bounded wait runs out (short limit)
  int* d_err = nullptr;  // set to 1 by a kernel whose bounded wait for its input ran out
};

// Plain form (one thread per site, reference arithmetic order), plain.cu.
template <class T> void launch_stage1(const Group<T>& g, int par, cudaStream_t st);
template <class T> void launch_stage2(const Group<T>& g, int par, cudaStream_t st);
template <class T> void launch_div(const Group<T>& g, int par, cudaStream_t st);
template <class T> void launch_correct(const Group<T>& g, int par, cudaStream_t st);
// FP64 diagnostics: per-instance partials into d_inst[i].red (nblocks_out per instance).
template <class T> int launch_stats(const Group<T>& g, int par, cudaStream_t st, bool full = true);
int stats_partials_per_instance(int N);

// Poisson solve by FFT (fft.cu): W <- (inverse FFT of -FFT(W)/k^2) / N^3.
// pass 0: forward x; 1: forward y; 2: forward z, divide, inverse z; 3: inverse y; 4: inverse x + scale.
template <class T> void launch_fft_pass(const Group<T>& g, int pass, cudaStream_t st);
template <class T> size_t fft_smem_bytes(int N, int pass);
// Sets the dynamic shared-memory limits of the FFT kernels for size N (call before capture).
template <class T> void fft_prepare(int N);
// Stockham lines per CTA: the candidates for size N (largest first) and the one a group uses.
template <class T> std::vector<int> fft_lb_candidates(int N);
template <class T> int fft_lines(const Group<T>& g);
// Register-resident FFT passes (fftreg_*.cu): false when the size has none (Stockham is used).
template <class T> bool fftreg_launch(const Group<T>& g, int pass, cudaStream_t st);
template <class T> void fftreg_prepare(int N);
// Fills the register FFT's __constant__ twiddle table of size N on the current device (its
// kernels read it; call once per device and size before they run; allocates nothing).
template <class T> void fftreg_twiddles(int N);
template <class T> bool fftreg_has(int N);
// Forward x + y (dir 0) or inverse y + x (dir 1) of every z-plane, one CTA per plane (fft_kind 2):
// false when the group does not use it.
template <class T> bool fftreg_plane_launch(const Group<T>& g, int dir, cudaStream_t st);
// The staged z pass of size N (FP32): builds the descriptors of the complex fields W[i] in a new
// device array (*d_maps, caller frees) and returns the persistent grid; 0 when N has none.
int fftreg_zt_setup(int N, const std::vector<const void*>& W, void** d_maps);

// Fused FP32 form (fused.cu): rhs (u*, P*, phi'), div (packed Poisson source), correct (u, P).
void launch_fused_rhs(const Group<float>& g, int par, cudaStream_t st);
void launch_fused_div(const Group<float>& g, int par, cudaStream_t st);
void launch_fused_correct(const Group<float>& g, int par, cudaStream_t st);
bool fused_supported(int N);
// Sets the fused kernels' dynamic shared-memory limits (call before capture).
void fused_prepare();

// readDraw.py reductions (post.cu): centroid partials (centroid_blocks() x 4 doubles) and the
// 9 slice planes of N*N doubles at z = zs.
// FP64 <-> FP32 field conversion on the device (post.cu): dst[i] = src[i] and
// dst[i] = src[i * stride] * scale (an exact power of two).
void launch_to_f32(const double* src, float* dst, size_t n, cudaStream_t st);
// scale_bits: the float bits of the maximum whose power of two (pow2_denorm) scales the values
// (device memory; nullptr: no scaling)
void launch_to_f64(const float* src, size_t stride, double* dst, size_t n, const int* scale_bits, cudaStream_t st);
void launch_gather_f64(const double* src, size_t stride, double* dst, size_t n, cudaStream_t st);
// The fused FP32 form's compensated fields (post.cu): an FP64 field split into its FP32 value and
// the remainder (bf16 lo or FP32 lo32), and joined back; hi and lo strided (2: one half of a pair
// field).
void launch_split(const double* src, float* hi, __nv_bfloat16* lo, float* lo32, size_t n, int stride, cudaStream_t st);
void launch_join(const float* hi, const __nv_bfloat16* lo, const float* lo32, double* dst, size_t n, int stride,
                 cudaStream_t st);
int centroid_blocks();
template <class T> void launch_centroid(const InstDev<T>* d_all, int inst, int par, double* part, cudaStream_t st);
template <class T>
void launch_slice(const InstDev<T>* d_all, int inst, int par, int N, int zs, double* out, cudaStream_t st);

}  // namespace ttsh
