// noalloc.cu — ttsh_step_noalloc: the FP64 step of one small droplet on caller-owned device
// buffers, with all working memory in one fixed device array of this library.
//
// Who needs it: callers whose device memory is owned by someone else, so that they cannot (or
// must not) call cudaMalloc/cudaFree themselves or through this library. Examples are a host
// application whose allocator has already reserved the GPU's memory (a cudaMalloc from a
// second allocator fails or fragments it), jobs run under a per-process device-memory cap,
// and loops that cannot afford cudaFree, which waits for all work on the device to finish.
// Such callers pass their own input/output arrays; everything else this step needs lives in
// g_noalloc_scratch below.
//
// Limits and sharing:
//   * N <= TTSH_NOALLOC_MAX_N (32), FP64 only. The scratch array is
//     22 * 32^3 * 8 bytes + 64 KiB (about 5.8 MB) and exists on every GPU that loads
//     libttsh.so until the process exits.
//   * Every call uses the same array and leaves its contents behind; nothing in it has to start
//     at zero (each step writes every scratch word it later reads). Calls whose GPU work
//     overlaps — on two streams, or from two host threads — race on the array: serialise them.
//   * The first call on a device looks up the array's device address (cudaGetSymbolAddress,
//     with that device current); the first call for a size on a device sets the FFT kernels'
//     shared-memory limits and fills the register FFT's constant twiddle table, then waits for
//     the device to finish (that table is written through the legacy stream, which a caller's
//     non-blocking stream does not wait for). Make those first calls before any stream capture
//     is started on the calling thread.
//   * Every later call only enqueues work on the caller's stream: the tables and the droplet
//     descriptor travel as the parameter of a small set-up kernel (copied at launch), not through
//     host memory that a copy would have to wait for or outlive.
// The step kernels are the plain-form kernels of plain.cu and fft.cu, unchanged.
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <mutex>
#include <stdexcept>
#include <string>

#include "../../include/ttsh.h"
#include "common.cuh"
#include "internal.h"
#include "kernels.h"

namespace {

constexpr int kMaxN = TTSH_NOALLOC_MAX_N;
constexpr size_t kN3 = (size_t)kMaxN * kMaxN * kMaxN;
constexpr size_t kField = kN3 * sizeof(double);
// 20 real scratch fields (mu_0, mu_b x3, sigma_ab x9, phi', u*' x3, P*' x3) + the complex W (2).
constexpr size_t kFieldsBytes = 22 * kField;
constexpr size_t kTailBytes = 64 * 1024;  // tables and the instance descriptor
constexpr size_t kScratchBytes = kFieldsBytes + kTailBytes;

const double kPi = 3.1415926535897932384626433832795;

}  // namespace

// The fixed working memory (device side). Host code must not pass this name to a kernel: on
// the host it is only a stand-in for the symbol; the device address comes from
// cudaGetSymbolAddress (noalloc_scratch_address below).
static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

namespace {

std::mutex g_mu;
void* g_addr[256] = {nullptr};
bool g_prepared[256][kMaxN + 1] = {{false}};

int fail(int code, const std::string& msg) { return ttsh::set_error(code, "ttsh_step_noalloc: " + msg); }

// What one call writes into the tail of the working array before its steps: the droplet
// descriptor, the twiddles exp(-2 pi i k / N) and the wavenumber tables (k, k^2, sin(k h)/h,
// (2 + cos(k h))/3), passed by value as a kernel parameter (about 2 KB, within the 4 KB limit).
struct Setup {
  ttsh::InstDev<double> inst;
  double2 tw[kMaxN];
  double tab[4 * kMaxN];
};
static_assert(sizeof(Setup) <= 4000, "set-up parameter within the kernel parameter limit");

__global__ void k_noalloc_setup(const Setup s, ttsh::InstDev<double>* d_inst, double2* d_tw, double* d_tab) {
  for (int i = threadIdx.x; i < kMaxN; i += blockDim.x) d_tw[i] = s.tw[i];
  for (int i = threadIdx.x; i < 4 * kMaxN; i += blockDim.x) d_tab[i] = s.tab[i];
  if (threadIdx.x == 0) *d_inst = s.inst;
}

// Once per device (that device current): the device address of g_noalloc_scratch.
int noalloc_scratch_address(int dev, unsigned char** out) {
  std::lock_guard<std::mutex> lk(g_mu);
  if (dev < 0 || dev >= 256) return fail(TTSH_E_UNSUPPORTED, "device index >= 256");
  if (!g_addr[dev]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return fail(TTSH_E_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
    g_addr[dev] = p;
  }
  *out = static_cast<unsigned char*>(g_addr[dev]);
  return TTSH_OK;
}

bool factors_ok(int N) {
  int m = N;
  for (int p : {2, 3, 5})
    while (m % p == 0) m /= p;
  return m == 1;
}

}  // namespace

extern "C" int ttsh_step_noalloc(const ttsh_input* in, const ttsh_ext* ext, int nsteps, double* phi, double* P,
                                 double* u, double* ustar, double* Pstar, double* p_v, double* p_p, void* stream) {
  using namespace ttsh;
  if (!in || !ext || !phi || !P || !u || !ustar || !Pstar || !p_v || !p_p || nsteps < 0)
    return fail(TTSH_E_INVALID, "null argument or negative step count");
  if (in->ReadSuccess != TTSH_READ_SUCCESS) return fail(TTSH_E_PARSE, "input: ReadSuccess != -8848");
  const int N = in->Nx;
  if (in->Ny != N || in->Nz != N) return fail(TTSH_E_UNSUPPORTED, "grid must be cubic");
  if (N < 8 || N > kMaxN)
    return fail(TTSH_E_UNSUPPORTED, "N = " + std::to_string(N) + " is outside [8, " + std::to_string(kMaxN) +
                                        "], the size of the fixed working memory");
  if (!factors_ok(N)) return fail(TTSH_E_UNSUPPORTED, "N must factor into 2, 3, 5");
  if (ext->precision != 64) return fail(TTSH_E_UNSUPPORTED, "FP64 only");
  if (ext->k2_mode != 0 && ext->k2_mode != 1) return fail(TTSH_E_INVALID, "k2_mode must be 0 or 1");
  if (!(in->h > 0) || !(in->dt0 > 0)) return fail(TTSH_E_INVALID, "h and dt0 must be > 0");
  if (in->TimeScheme != 1) return fail(TTSH_E_UNSUPPORTED, "only TimeScheme 1 (explicit Euler)");

  cudaStream_t st = static_cast<cudaStream_t>(stream);
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return fail(TTSH_E_NODEVICE, cudaGetErrorString(e));
  unsigned char* base = nullptr;
  int rc = noalloc_scratch_address(dev, &base);
  if (rc) return rc;
  try {
    {
      std::lock_guard<std::mutex> lk(g_mu);
      if (!g_prepared[dev][N]) {
        fft_prepare<double>(N);
        if (fftreg_has<double>(N)) fftreg_twiddles<double>(N);  // the register FFT's constant table
        // the table copy runs on the legacy stream: let it land before kernels on any stream read it
        const cudaError_t es = cudaDeviceSynchronize();
        if (es != cudaSuccess) throw std::runtime_error(std::string("first-call set-up: ") + cudaGetErrorString(es));
        g_prepared[dev][N] = true;
      }
    }
    const size_t n = (size_t)N * N * N;
    // carve the scratch: fields first (each sized for N), then tables, then the descriptor
    double* f = reinterpret_cast<double*>(base);
    Setup su{};
    InstDev<double>& I = su.inst;
    size_t off = 0;
    auto take = [&](size_t count) { double* p = f + off; off += count; return p; };
    I.mu0 = take(n);
    for (int b = 0; b < 3; ++b) I.mu[b] = take(n);
    for (int b = 0; b < 9; ++b) I.sig[b] = take(n);
    double* phi_new = take(n);
    double* us_new = take(3 * n);
    double* ps_new = take(3 * n);
    I.W = reinterpret_cast<double2*>(take(2 * n));
    unsigned char* tail = base + kFieldsBytes;
    double2* d_tw = reinterpret_cast<double2*>(tail);
    double* d_kval = reinterpret_cast<double*>(tail + 8192);
    double* d_k2t = d_kval + kMaxN;
    double* d_St = d_k2t + kMaxN;
    double* d_Ct = d_St + kMaxN;
    InstDev<double>* d_inst = reinterpret_cast<InstDev<double>*>(tail + 32768);

    // the same tables and constants as ttsh_create builds (api.cu)
    const double h = in->h;
    for (int k = 0; k < N; ++k) {
      const double a = -2.0 * kPi * (double)k / (double)N;
      su.tw[k] = make_double2(std::cos(a), std::sin(a));
      double kk = 2 * kPi * k / (N * h + 0.0);
      if (k >= N / 2) kk = 2 * kPi * (k - N) / (N * h + 0.0);
      su.tab[k] = kk;
      su.tab[kMaxN + k] = kk * kk;
      su.tab[2 * kMaxN + k] = std::sin(kk * h) / h;
      su.tab[3 * kMaxN + k] = (2.0 + std::cos(kk * h)) / 3.0;
    }
    I.N = N;
    I.stale = (ext->quirks & TTSH_QUIRK_STALE_HALO) ? 1 : 0;
    I.k2mode = ext->k2_mode;
    int m = N, ns = 0;
    while (m % 4 == 0) { I.radix[ns++] = 4; m /= 4; }
    while (m % 2 == 0) { I.radix[ns++] = 2; m /= 2; }
    while (m % 3 == 0) { I.radix[ns++] = 3; m /= 3; }
    while (m % 5 == 0) { I.radix[ns++] = 5; m /= 5; }
    I.nstages = ns;
    Phys<double>& p = I.ph;
    p.h = h; p.dt = in->dt0; p.inv_dt = 1.0 / in->dt0; p.dt_d = in->dt0;
    p.mu = in->mu; p.cA = in->cA; p.alpha = in->alpha; p.beta = in->beta; p.eta = in->eta;
    p.La2 = in->La * in->La; p.kappa = in->kappa; p.lambda0 = in->lambda0; p.aPhi2 = in->aPhi * 2;
    p.kPhi = in->kPhi; p.gamma = in->gamma; p.A = in->A; p.zeta = ext->zeta;
    p.c2h = 1.0 / (2.0 * h); p.cl12 = 1.0 / (12 * h * h); p.cl23 = 2.0 / (3 * h * h); p.cl143 = 14.0 / (3 * h * h);
    p.invN3 = 1.0 / ((double)N * N * N);
    I.phi[0] = phi; I.phi[1] = phi_new;
    for (int b = 0; b < 3; ++b) {
      I.P[b] = P + b * n;
      I.U[b] = u + b * n;
      I.Us[0][b] = ustar + b * n; I.Us[1][b] = us_new + b * n;
      I.Ps[0][b] = Pstar + b * n; I.Ps[1][b] = ps_new + b * n;
    }
    I.tw = d_tw; I.kval = d_kval; I.k2t = d_k2t; I.St = d_St; I.Ct = d_Ct;
    I.red = nullptr;
#define NA_CK(call)                                                                 \
  do {                                                                              \
    cudaError_t e_ = (call);                                                        \
    if (e_ != cudaSuccess) throw std::runtime_error(std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)
    // descriptor and tables into the working array, in stream order, by value (no host copy)
    k_noalloc_setup<<<1, 128, 0, st>>>(su, d_inst, d_tw, d_kval);
    NA_CK(cudaGetLastError());
    Group<double> g{d_inst, 1, N};
    for (int t = 0; t < nsteps; ++t) {
      launch_stage1<double>(g, 0, st);
      launch_stage2<double>(g, 0, st);
      launch_div<double>(g, 0, st);
      for (int pass = 0; pass < 5; ++pass) launch_fft_pass<double>(g, pass, st);
      launch_correct<double>(g, 0, st);
      // the new phi, u*, P* become the caller's state (u*, P* feed the next step's stale halo)
      NA_CK(cudaMemcpyAsync(phi, phi_new, n * sizeof(double), cudaMemcpyDeviceToDevice, st));
      NA_CK(cudaMemcpyAsync(ustar, us_new, 3 * n * sizeof(double), cudaMemcpyDeviceToDevice, st));
      NA_CK(cudaMemcpyAsync(Pstar, ps_new, 3 * n * sizeof(double), cudaMemcpyDeviceToDevice, st));
    }
    if (nsteps > 0) {
      // pressures: real and imaginary parts of the packed field W
      NA_CK(cudaMemcpy2DAsync(p_v, sizeof(double), I.W, 2 * sizeof(double), sizeof(double), n,
                              cudaMemcpyDeviceToDevice, st));
      NA_CK(cudaMemcpy2DAsync(p_p, sizeof(double), reinterpret_cast<double*>(I.W) + 1, 2 * sizeof(double),
                              sizeof(double), n, cudaMemcpyDeviceToDevice, st));
    }
    NA_CK(cudaGetLastError());
#undef NA_CK
  } catch (const std::exception& ex) {
    return fail(TTSH_E_CUDA, ex.what());
  }
  return TTSH_OK;
}
