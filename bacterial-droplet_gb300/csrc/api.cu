// api.cu — libttsh host runtime and C ABI (declared in include/ttsh.h).
//
// Device memory: one arena per droplet holding its unpadded N^3 fields
// (phi x2, P, u, u* x2, P* x2, the packed complex Poisson field, and in the plain
// form the mu_0, mu_b, sigma_ab intermediates) plus its small tables (twiddles,
// wavenumbers). Droplets of equal N form a group; every kernel of the step is
// launched once per group, covering all droplets of the group. The whole step
// (all groups) is captured into a CUDA graph per parity of the ping-pong buffers.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <stdexcept>
#include <thread>
#include <string>
#include <type_traits>
#include <vector>

#include "../../include/ttsh.h"
#include "common.cuh"
#include "internal.h"
#include "kernels.h"

namespace ttsh {

static thread_local std::string g_last_error;

int set_error(int code, const std::string& msg) {
  g_last_error = msg;
  return code;
}

struct CudaError : std::runtime_error {
  using std::runtime_error::runtime_error;
};

#define CK(call)                                                                                     \
  do {                                                                                               \
    cudaError_t e_ = (call);                                                                         \
    if (e_ != cudaSuccess)                                                                           \
      throw CudaError(std::string(#call) + ": " + cudaGetErrorString(e_));                          \
  } while (0)

namespace {

const double kPi = 3.1415926535897932384626433832795;  // TTSH3D.cu:27

std::vector<int> radix_plan(int N) {
  std::vector<int> r;
  int m = N;
  while (m % 4 == 0) { r.push_back(4); m /= 4; }
  while (m % 2 == 0) { r.push_back(2); m /= 2; }
  while (m % 3 == 0) { r.push_back(3); m /= 3; }
  while (m % 5 == 0) { r.push_back(5); m /= 5; }
  if (m != 1) r.clear();
  return r;
}

// Kernel classes reported by ttsh_profile_kernels.
enum KClass { K_STAGE1, K_STAGE2, K_DIV, K_FFT0, K_FFT1, K_FFT2, K_FFT3, K_FFT4, K_CORRECT, K_FUSED_RHS,
              K_FUSED_DIV, K_FUSED_CORRECT, K_FFT_XY, K_FFT_YX, K_NCLASS };
const char* kNames[K_NCLASS] = {"stage1", "stage2", "div", "fft_x_fwd", "fft_y_fwd", "fft_z_poisson", "fft_y_inv",
                                "fft_x_inv", "correct", "fused_rhs", "fused_div", "fused_correct",
                                "fft_xy_fwd", "fft_yx_inv"};

// The Poisson solve of a group: x+y per plane, z, y+x per plane (fft_kind 2 with a register
// kernel for the size), else one launch per axis pass. `run(class, launch)` wraps each launch.
template <class T, class R>
void enqueue_fft(const Group<T>& g, cudaStream_t st, R&& run) {
  if (g.fft_kind == 2 && fftreg_has<T>(g.N)) {
    run(K_FFT_XY, [&] { fftreg_plane_launch<T>(g, 0, st); });
    run(K_FFT2, [&] { launch_fft_pass<T>(g, 2, st); });
    run(K_FFT_YX, [&] { fftreg_plane_launch<T>(g, 1, st); });
  } else {
    for (int pass = 0; pass < 5; ++pass) run(K_FFT0 + pass, [&] { launch_fft_pass<T>(g, pass, st); });
  }
}
template <class T>
int fft_launches(const Group<T>& g) { return (g.fft_kind == 2 && fftreg_has<T>(g.N)) ? 3 : 5; }

struct Prof {
  cudaStream_t st;
  std::vector<std::pair<int, std::pair<cudaEvent_t, cudaEvent_t>>> ev;
  void begin(int cls) {
    cudaEvent_t a, b;
    CK(cudaEventCreate(&a));
    CK(cudaEventCreate(&b));
    CK(cudaEventRecord(a, st));
    ev.push_back({cls, {a, b}});
  }
  void end() { CK(cudaEventRecord(ev.back().second.second, st)); }
};

struct InstHost {
  int N = 0;
  ttsh_input in{};
  ttsh_ext ext{};
  double T = 0;
  void* arena = nullptr;
};

template <class T>
struct Engine {
  std::vector<InstDev<T>> h;     // host copies of the device descriptors
  std::vector<Group<T>> groups;  // device descriptor arrays
  std::vector<int> grp, loc;     // instance -> group, index in group
  std::vector<std::vector<int>> members;

  void free_all() {
    for (auto& g : groups)
      if (g.d_inst) cudaFree(g.d_inst);
    groups.clear();
  }

  void enqueue_step(int par, cudaStream_t st, bool fused, Prof* pr) {
    for (auto& g : groups) {
      auto run = [&](int cls, auto&& fn) {
        if (pr) pr->begin(cls);
        fn();
        if (pr) pr->end();
      };
      if (fused) {
        run(K_FUSED_RHS, [&] { launch_fused_rhs_t(g, par, st); });
        run(K_FUSED_DIV, [&] { launch_fused_div_t(g, par, st); });
      } else {
        run(K_STAGE1, [&] { launch_stage1<T>(g, par, st); });
        run(K_STAGE2, [&] { launch_stage2<T>(g, par, st); });
        run(K_DIV, [&] { launch_div<T>(g, par, st); });
      }
      enqueue_fft(g, st, run);
      if (fused) run(K_FUSED_CORRECT, [&] { launch_fused_correct_t(g, par, st); });
      else run(K_CORRECT, [&] { launch_correct<T>(g, par, st); });
    }
  }
  void launch_fused_rhs_t(const Group<T>& g, int par, cudaStream_t st);
  void launch_fused_div_t(const Group<T>& g, int par, cudaStream_t st);
  void launch_fused_correct_t(const Group<T>& g, int par, cudaStream_t st);
  int launches(bool fused) const {
    int n = 0;
    for (const auto& g : groups) n += (fused ? 3 : 4) + fft_launches(g);
    return n;
  }
};

template <>
void Engine<float>::launch_fused_rhs_t(const Group<float>& g, int par, cudaStream_t st) { launch_fused_rhs(g, par, st); }
template <>
void Engine<float>::launch_fused_div_t(const Group<float>& g, int par, cudaStream_t st) { launch_fused_div(g, par, st); }
template <>
void Engine<float>::launch_fused_correct_t(const Group<float>& g, int par, cudaStream_t st) {
  launch_fused_correct(g, par, st);
}
template <>
void Engine<double>::launch_fused_div_t(const Group<double>&, int, cudaStream_t) {
  throw std::runtime_error("fused form is FP32 only");
}
template <>
void Engine<double>::launch_fused_rhs_t(const Group<double>&, int, cudaStream_t) {
  throw std::runtime_error("fused form is FP32 only");
}
template <>
void Engine<double>::launch_fused_correct_t(const Group<double>&, int, cudaStream_t) {
  throw std::runtime_error("fused form is FP32 only");
}

}  // namespace
}  // namespace ttsh

using namespace ttsh;

struct ttsh_sim {
  int device = 0;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  int precision = 64;
  bool fused = false;
  std::vector<InstHost> inst;
  Engine<float> ef;
  Engine<double> ed;
  int par = 0;
  int64_t steps = 0;
  cudaGraphExec_t gexec[2] = {nullptr, nullptr};
  std::vector<void*> tables;  // shared per-N tables
  double* post = nullptr;     // snapshot-reduction scratch (allocated on first use)
  size_t post_bytes = 0;
  int* d_err = nullptr;       // device word set by a kernel whose bounded wait ran out
  // the asynchronous snapshot writer: one page-locked buffer (u, P, phi in FP64) that the device
  // fills in stream order, and the host thread that formats it
  double* conf_buf = nullptr;
  size_t conf_cap = 0;
  cudaEvent_t conf_ready = nullptr;
  std::thread conf_thread;
  int conf_rc = 0;
  std::string conf_msg;

  template <class F>
  void with_engine(F&& f) {
    if (precision == 32) f(ef);
    else f(ed);
  }
};

namespace {

// Validation of one droplet's parameters; returns 0 or sets the error.
int validate(const ttsh_input& in, const ttsh_ext& ext) {
  if (in.ReadSuccess != TTSH_READ_SUCCESS) return set_error(TTSH_E_PARSE, "input: ReadSuccess != -8848");
  if (in.Nx != in.Ny || in.Ny != in.Nz)
    return set_error(TTSH_E_UNSUPPORTED, "grid must be cubic (the reference's FFT plan, TTSH3D.cu:1123)");
  if (in.Nx < 8 || in.Nx > 1024) return set_error(TTSH_E_UNSUPPORTED, "N must be in [8, 1024]");
  if (radix_plan(in.Nx).empty()) return set_error(TTSH_E_UNSUPPORTED, "N must factor into 2, 3, 5");
  if (!(in.h > 0) || !(in.dt0 > 0)) return set_error(TTSH_E_INVALID, "h and dt0 must be > 0");
  if (in.TimeScheme != 1)
    return set_error(TTSH_E_UNSUPPORTED, "only TimeScheme 1 (explicit Euler) exists in the reference step");
  if (ext.precision != 32 && ext.precision != 64) return set_error(TTSH_E_INVALID, "precision must be 32 or 64");
  if (ext.k2_mode != 0 && ext.k2_mode != 1) return set_error(TTSH_E_INVALID, "k2_mode must be 0 or 1");
  return TTSH_OK;
}

template <class T>
Phys<T> make_phys(const ttsh_input& in, const ttsh_ext& ext) {
  Phys<T> p{};
  const double h = in.h;
  p.h = (T)h;
  p.dt = (T)in.dt0;
  p.inv_dt = (T)(1.0 / in.dt0);
  p.dt_d = in.dt0;
  p.mu = (T)in.mu; p.cA = (T)in.cA; p.alpha = (T)in.alpha; p.beta = (T)in.beta; p.eta = (T)in.eta;
  p.La2 = (T)(in.La * in.La);
  p.kappa = (T)in.kappa; p.lambda0 = (T)in.lambda0;
  p.aPhi2 = (T)(in.aPhi * 2);
  p.kPhi = (T)in.kPhi; p.gamma = (T)in.gamma; p.A = (T)in.A; p.zeta = (T)ext.zeta;
  p.c2h = (T)(1.0 / (2.0 * h));
  p.cl12 = (T)(1.0 / (12 * h * h));
  p.cl23 = (T)(2.0 / (3 * h * h));
  p.cl143 = (T)(14.0 / (3 * h * h));
  p.clz = (T)(1.0 / (h * h));
  const double n3 = (double)in.Nx * in.Nx * in.Nx;
  p.invN3 = (T)(1.0 / n3);
  return p;
}

size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

template <class T>
void build_engine(ttsh_sim* s, Engine<T>& E) {
  typedef typename CxT<T>::type C;
  const int n = (int)s->inst.size();
  E.h.resize(n);
  E.grp.resize(n);
  E.loc.resize(n);
  std::map<int, int> by_n;
  for (int i = 0; i < n; ++i) {
    const int N = s->inst[i].N;
    if (!by_n.count(N)) {
      by_n[N] = (int)E.members.size();
      E.members.push_back({});
    }
    E.grp[i] = by_n[N];
    E.loc[i] = (int)E.members[E.grp[i]].size();
    E.members[E.grp[i]].push_back(i);
  }
  // per-N tables
  std::map<int, InstDev<T>> tab;
  for (auto& kv : by_n) {
    const int N = kv.first;
    const double h = s->inst[E.members[kv.second][0]].in.h;
    std::vector<C> tw(N);
    std::vector<double> kval(N);
    std::vector<T> k2t(N), St(N), Ct(N);
    for (int k = 0; k < N; ++k) {
      const double a = -2.0 * kPi * (double)k / (double)N;
      tw[k].x = (T)std::cos(a);
      tw[k].y = (T)std::sin(a);
      // initPoissonSolver (TTSH3D.cu:1093-1117)
      double kk = 2 * kPi * k / (N * h + 0.0);
      if (k >= N / 2) kk = 2 * kPi * (k - N) / (N * h + 0.0);
      kval[k] = kk;
      k2t[k] = (T)(kk * kk);
      St[k] = (T)(std::sin(kk * h) / h);
      Ct[k] = (T)((2.0 + std::cos(kk * h)) / 3.0);
    }
    size_t bytes = align256(N * sizeof(C)) + align256(N * sizeof(double)) + 3 * align256(N * sizeof(T));
    char* d = nullptr;
    CK(cudaMalloc(&d, bytes));
    s->tables.push_back(d);
    InstDev<T> t{};
    size_t off = 0;
    t.tw = reinterpret_cast<C*>(d + off); CK(cudaMemcpy(d + off, tw.data(), N * sizeof(C), cudaMemcpyHostToDevice));
    off += align256(N * sizeof(C));
    t.kval = reinterpret_cast<double*>(d + off);
    CK(cudaMemcpy(d + off, kval.data(), N * sizeof(double), cudaMemcpyHostToDevice));
    off += align256(N * sizeof(double));
    t.k2t = reinterpret_cast<T*>(d + off); CK(cudaMemcpy(d + off, k2t.data(), N * sizeof(T), cudaMemcpyHostToDevice));
    off += align256(N * sizeof(T));
    t.St = reinterpret_cast<T*>(d + off); CK(cudaMemcpy(d + off, St.data(), N * sizeof(T), cudaMemcpyHostToDevice));
    off += align256(N * sizeof(T));
    t.Ct = reinterpret_cast<T*>(d + off); CK(cudaMemcpy(d + off, Ct.data(), N * sizeof(T), cudaMemcpyHostToDevice));
    tab[N] = t;
    fft_prepare<T>(N);
    if (fftreg_has<T>(N)) fftreg_twiddles<T>(N);
  }
  // per-instance arenas
  for (int i = 0; i < n; ++i) {
    InstHost& ih = s->inst[i];
    const int N = ih.N;
    const size_t nn = (size_t)N * N * N;
    const size_t fb = align256(nn * sizeof(T));
    // phi x2, P, u, u* x2, P* x2, the packed Poisson field W, and: fused, the phi compensation,
    // the bf16 compensations of u (3) and the bf16 pairs compensating u*, P* x2 (6 FP32 slots);
    // plain, the 13 intermediates
    const int nfields = 2 + 3 + 3 + 6 + 6 + (s->fused ? 1 + 6 : 13);
    const size_t lb = align256(nn * sizeof(__nv_bfloat16));
    const size_t bytes = nfields * fb + align256(nn * sizeof(C)) + (s->fused ? 3 * lb : 0);
    char* d = nullptr;
    cudaError_t e = cudaMalloc(&d, bytes);
    if (e != cudaSuccess) throw std::bad_alloc();
    ih.arena = d;
    CK(cudaMemset(d, 0, bytes));
    InstDev<T>& I = E.h[i];
    I = tab[N];
    I.N = N;
    I.stale = (ih.ext.quirks & TTSH_QUIRK_STALE_HALO) ? 1 : 0;
    I.k2mode = ih.ext.k2_mode;
    std::vector<int> r = radix_plan(N);
    I.nstages = (int)r.size();
    for (size_t k = 0; k < r.size(); ++k) I.radix[k] = r[k];
    I.ph = make_phys<T>(ih.in, ih.ext);
    size_t off = 0;
    auto take = [&]() { T* p = reinterpret_cast<T*>(d + off); off += fb; return p; };
    I.phi[0] = take(); I.phi[1] = take();
    for (int b = 0; b < 3; ++b) I.P[b] = take();
    for (int b = 0; b < 3; ++b) I.U[b] = take();
    if (s->fused) {
      // u*, P* as pairs (u*_b, P*_b), two FP32 slots each (the same 12 slots as Us, Ps x2), in
      // parity order: star[q] holds 3 consecutive pair fields (they double as the FP64 scratch
      // of the host interface, 3 FP64 fields)
      for (int q = 0; q < 2; ++q)
        for (int b = 0; b < 3; ++b) {
          I.star[q][b] = reinterpret_cast<float2*>(d + off);
          off += 2 * fb;
        }
      I.phic = take();
      auto take_b = [&]() { __nv_bfloat16* p = reinterpret_cast<__nv_bfloat16*>(d + off); off += lb; return p; };
      for (int f = 0; f < 3; ++f) I.lo[f] = take_b();
      for (int q = 0; q < 2; ++q)
        for (int b = 0; b < 3; ++b) I.starlo[q][b] = reinterpret_cast<__nv_bfloat162*>(take());
    } else {
      for (int q = 0; q < 2; ++q)
        for (int b = 0; b < 3; ++b) I.Us[q][b] = take();
      for (int q = 0; q < 2; ++q)
        for (int b = 0; b < 3; ++b) I.Ps[q][b] = take();
    }
    if (!s->fused) {
      I.mu0 = take();
      for (int b = 0; b < 3; ++b) I.mu[b] = take();
      for (int b = 0; b < 9; ++b) I.sig[b] = take();
    }
    I.W = reinterpret_cast<C*>(d + off);
  }
  if constexpr (std::is_same<T, float>::value) {
    // per droplet: the maxima of the packed Poisson source (two ints, for its balancing) and, in
    // the fused form, of u*, P* (two ints, the grid of the exact divergence)
    int* wm = nullptr;
    CK(cudaMalloc(&wm, 4 * sizeof(int) * (size_t)n));
    CK(cudaMemset(wm, 0, 4 * sizeof(int) * (size_t)n));
    s->tables.push_back(wm);
    for (int i = 0; i < n; ++i) {
      E.h[i].wmax = wm + 4 * i;
      if (s->fused) E.h[i].smax = wm + 4 * i + 2;
    }
  }
  if (!s->d_err) {
    CK(cudaMalloc(&s->d_err, sizeof(int)));
    CK(cudaMemset(s->d_err, 0, sizeof(int)));
    s->tables.push_back(s->d_err);
  }
  for (size_t g = 0; g < E.members.size(); ++g) {
    // FP64 diagnostics partials of all droplets of the group, contiguous (one copy back)
    const size_t per = 4 * (size_t)stats_partials_per_instance(0);
    double* red = nullptr;
    CK(cudaMalloc(&red, per * E.members[g].size() * sizeof(double)));
    s->tables.push_back(red);
    for (size_t k = 0; k < E.members[g].size(); ++k) E.h[E.members[g][k]].red = red + k * per;
    Group<T> G{};
    G.red = red;
    // TTSH_FFT="stockham": shared-memory Stockham passes only; "separate": register passes, one
    // launch per axis; otherwise register kernels with x and y of a plane in one launch
    const char* fk = std::getenv("TTSH_FFT");
    G.fft_kind = (fk && std::string(fk) == "stockham") ? 1 : ((fk && std::string(fk) == "separate") ? 0 : 2);
    G.n = (int)E.members[g].size();
    G.N = s->inst[E.members[g][0]].N;
    G.d_err = s->d_err;
    // FP32, on request (TTSH_ZTMA=1): the z pass with its input staged by the tensor memory
    // accelerator where the size has it; by default the z pass loads its input directly (faster
    // since its twiddles come from constant memory)
    const char* zt = std::getenv("TTSH_ZTMA");
    if (std::is_same<T, float>::value && zt && std::string(zt) == "1") {
      std::vector<const void*> W;
      for (int i : E.members[g]) W.push_back(E.h[i].W);
      void* maps = nullptr;
      G.zt_grid = fftreg_zt_setup(G.N, W, &maps);
      if (maps) s->tables.push_back(maps);
      G.d_tmz = maps;
      // failure test only: every CTA skips its first copy and its wait for it runs out
      const char* drop = std::getenv("TTSH_TEST_DROP_STAGED_COPY");
      G.zt_drop = (drop && std::string(drop) == "1") ? 1 : 0;
    }
    std::vector<InstDev<T>> arr;
    for (int i : E.members[g]) arr.push_back(E.h[i]);
    CK(cudaMalloc(&G.d_inst, sizeof(InstDev<T>) * arr.size()));
    CK(cudaMemcpy(G.d_inst, arr.data(), sizeof(InstDev<T>) * arr.size(), cudaMemcpyHostToDevice));
    E.groups.push_back(G);
  }
  // the arena memsets ran on the legacy stream, which the non-blocking step stream does not wait for
  CK(cudaDeviceSynchronize());
}

void capture_graphs(ttsh_sim* s) {
  for (int q = 0; q < 2; ++q) {
    if (s->gexec[q]) { cudaGraphExecDestroy(s->gexec[q]); s->gexec[q] = nullptr; }
    cudaGraph_t g = nullptr;
    CK(cudaStreamBeginCapture(s->stream, cudaStreamCaptureModeRelaxed));
    try {
      s->with_engine([&](auto& E) { E.enqueue_step(q, s->stream, s->fused, nullptr); });
    } catch (...) {
      cudaStreamEndCapture(s->stream, &g);
      if (g) cudaGraphDestroy(g);
      throw;
    }
    CK(cudaStreamEndCapture(s->stream, &g));
    CK(cudaGraphInstantiate(&s->gexec[q], g, 0));
    CK(cudaGraphDestroy(g));
  }
}

void release(ttsh_sim* s) {
  if (!s) return;
  cudaSetDevice(s->device);
  if (s->conf_thread.joinable()) s->conf_thread.join();
  if (s->conf_buf) cudaFreeHost(s->conf_buf);
  if (s->conf_ready) cudaEventDestroy(s->conf_ready);
  if (s->stream) cudaStreamSynchronize(s->stream);
  for (int q = 0; q < 2; ++q)
    if (s->gexec[q]) cudaGraphExecDestroy(s->gexec[q]);
  s->ef.free_all();
  s->ed.free_all();
  for (auto& ih : s->inst)
    if (ih.arena) cudaFree(ih.arena);
  for (void* p : s->tables) cudaFree(p);
  if (s->post) cudaFree(s->post);
  if (s->own_stream && s->stream) cudaStreamDestroy(s->stream);
  delete s;
}

// TTSH_E_CUDA when a kernel's bounded wait for its staged input ran out since the handle was
// created (the state is then invalid); call after the stream has been synchronised.
int kernel_error(ttsh_sim* s) {
  int e = 0;
  if (s->d_err) CK(cudaMemcpy(&e, s->d_err, sizeof(int), cudaMemcpyDeviceToHost));
  return e ? set_error(TTSH_E_CUDA, "a kernel's wait for its staged input timed out; the state is invalid") : TTSH_OK;
}

template <class F>
int guarded(F&& f) {
  try {
    return f();
  } catch (const CudaError& e) {
    return set_error(TTSH_E_CUDA, e.what());
  } catch (const std::bad_alloc&) {
    return set_error(TTSH_E_NOMEM, "allocation failed");
  } catch (const std::exception& e) {
    return set_error(TTSH_E_CUDA, e.what());
  }
}

bool fused_ok(const ttsh_sim* s) {
  if (s->precision != 32) return false;
  for (auto& ih : s->inst)
    if (!fused_supported(ih.N)) return false;
  return true;
}

// TTSH_FORM_* of the batch: 0 = plain, 1 = fused, -1 = fused requested but unsupported.
int pick_form(const ttsh_sim* s) {
  const int want = s->inst[0].ext.form;
  if (want == TTSH_FORM_PLAIN) return 0;
  if (want == TTSH_FORM_FUSED) return fused_ok(s) ? 1 : -1;
  return fused_ok(s) ? 1 : 0;
}


// ---- autotuner ---------------------------------------------------------------------------

// Radix orders of the Stockham plan: radix_plan's (radix 4 first) and its reverse.
std::vector<std::vector<int>> radix_orders(int N) {
  std::vector<std::vector<int>> r;
  const std::vector<int> a = radix_plan(N);
  r.push_back(a);
  const std::vector<int> b(a.rbegin(), a.rend());
  if (b != a) r.push_back(b);
  return r;
}

// Mean device time per call of `launch`: `reps` calls captured in a CUDA graph (no host launch
// gaps between them), best of 3 rounds after one warm-up round; `prep` runs before every round,
// outside the timed region.
template <class P, class F>
double time_graph(cudaStream_t st, int reps, P&& prep, F&& launch) {
  cudaGraph_t g = nullptr;
  CK(cudaStreamBeginCapture(st, cudaStreamCaptureModeRelaxed));
  try {
    for (int r = 0; r < reps; ++r) launch();
  } catch (...) {
    cudaStreamEndCapture(st, &g);
    if (g) cudaGraphDestroy(g);
    throw;
  }
  CK(cudaStreamEndCapture(st, &g));
  cudaGraphExec_t ge = nullptr;
  const cudaError_t ei = cudaGraphInstantiate(&ge, g, 0);
  cudaGraphDestroy(g);
  CK(ei);
  cudaEvent_t a = nullptr, b = nullptr;
  double best = 1e30;
  try {
    CK(cudaEventCreate(&a));
    CK(cudaEventCreate(&b));
    for (int round = 0; round < 4; ++round) {
      prep();
      CK(cudaEventRecord(a, st));
      CK(cudaGraphLaunch(ge, st));
      CK(cudaEventRecord(b, st));
      CK(cudaEventSynchronize(b));
      float ms = 0;
      CK(cudaEventElapsedTime(&ms, a, b));
      if (round > 0) best = std::min(best, (double)ms / reps);
    }
  } catch (...) {
    if (a) cudaEventDestroy(a);
    if (b) cudaEventDestroy(b);
    cudaGraphExecDestroy(ge);
    throw;
  }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  cudaGraphExecDestroy(ge);
  return best;
}

template <class T>
void upload_group(ttsh_sim* s, Engine<T>& E, size_t gi) {
  std::vector<InstDev<T>> arr;
  for (int i : E.members[gi]) arr.push_back(E.h[i]);
  CK(cudaMemcpyAsync(E.groups[gi].d_inst, arr.data(), sizeof(InstDev<T>) * arr.size(), cudaMemcpyHostToDevice,
                     s->stream));
  CK(cudaStreamSynchronize(s->stream));
}

template <class T>
void set_radix(ttsh_sim* s, Engine<T>& E, size_t gi, const std::vector<int>& r) {
  for (int i : E.members[gi]) {
    E.h[i].nstages = (int)r.size();
    for (size_t k = 0; k < r.size(); ++k) E.h[i].radix[k] = r[k];
  }
  upload_group(s, E, gi);
}

template <class T>
void get_tuning(const ttsh_sim* s, const Engine<T>& E, size_t gi, ttsh_tuning* t) {
  const Group<T>& G = E.groups[gi];
  const InstDev<T>& I = E.h[E.members[gi][0]];
  std::memset(t, 0, sizeof(*t));
  t->N = G.N;
  t->n = G.n;
  t->fft_kind = G.fft_kind;
  t->fft_lb = G.fft_lb;
  t->nstages = I.nstages;
  for (int k = 0; k < I.nstages; ++k) t->radix[k] = I.radix[k];
  for (int k = 0; k < 3; ++k) t->zc[k] = s->fused ? G.zc[k] : 0;
  for (int k = 0; k < 4; ++k) t->ms[k] = G.tuned_ms[k];
}

// Checks a configuration against what the kernels support; returns an error message or "".
template <class T>
std::string check_tuning(const ttsh_sim* s, const Group<T>& G, const ttsh_tuning& t) {
  if (t.N != G.N || t.n != G.n) return "tuning: N or group size differs from the group";
  if (t.fft_kind < 0 || t.fft_kind > 2) return "tuning: fft_kind must be 0, 1 or 2";
  if (t.fft_lb != 0) {
    const std::vector<int> c = fft_lb_candidates<T>(G.N);
    if (std::find(c.begin(), c.end(), t.fft_lb) == c.end()) return "tuning: unsupported Stockham lines per CTA";
  }
  if (t.nstages < 1 || t.nstages > 16) return "tuning: bad radix plan length";
  long prod = 1;
  for (int k = 0; k < t.nstages; ++k) {
    const int r = t.radix[k];
    if (r != 2 && r != 3 && r != 4 && r != 5) return "tuning: radix must be 2, 3, 4 or 5";
    prod *= r;
  }
  if (prod != G.N) return "tuning: radix plan does not multiply to N";
  if (s->fused)
    for (int k = 0; k < 3; ++k) {
      if (t.zc[k] == 0) continue;  // the persistent grid
      if (t.zc[k] < 1) return "tuning: z-planes per CTA must be >= 1, or 0 (persistent grid)";
      if ((long)((G.N + t.zc[k] - 1) / t.zc[k]) * G.n > 65535) return "tuning: grid too large";
    }
  return "";
}

template <class T>
void apply_tuning(ttsh_sim* s, Engine<T>& E, size_t gi, const ttsh_tuning& t) {
  Group<T>& G = E.groups[gi];
  G.fft_kind = t.fft_kind;
  G.fft_lb = t.fft_lb;
  for (int k = 0; k < 4; ++k) G.tuned_ms[k] = 0;
  if (s->fused)
    for (int k = 0; k < 3; ++k) G.zc[k] = t.zc[k];
  set_radix(s, E, gi, std::vector<int>(t.radix, t.radix + t.nstages));
}

// Copies of the arrays the trial launches overwrite at the current parity (u, P, the phi
// compensation, the pressures), restored after the trials.
template <class T>
struct TrialBackup {
  std::vector<std::pair<void*, size_t>> arrays;
  char* buf = nullptr;
  void save(ttsh_sim* s, Engine<T>& E, size_t gi) {
    for (int i : E.members[gi]) {
      InstDev<T>& I = E.h[i];
      const size_t n = (size_t)I.N * I.N * I.N;
      for (int b = 0; b < 3; ++b) arrays.push_back({I.U[b], n * sizeof(T)});
      for (int b = 0; b < 3; ++b) arrays.push_back({I.P[b], n * sizeof(T)});
      if (I.phic) arrays.push_back({I.phic, n * sizeof(T)});
      arrays.push_back({I.W, 2 * n * sizeof(T)});
      if (I.wmax) arrays.push_back({I.wmax, 2 * sizeof(int)});  // the pressures' scales
      if (I.smax) {  // the fused form's compensation of u and the grid of its next divergence
        arrays.push_back({I.smax, 2 * sizeof(int)});
        for (int f = 0; f < 3; ++f) arrays.push_back({I.lo[f], n * sizeof(__nv_bfloat16)});
      }
    }
    size_t tot = 0;
    for (auto& a : arrays) tot += a.second;
    CK(cudaMalloc(&buf, tot));
    size_t off = 0;
    for (auto& a : arrays) {
      CK(cudaMemcpyAsync(buf + off, a.first, a.second, cudaMemcpyDeviceToDevice, s->stream));
      off += a.second;
    }
  }
  void restore(ttsh_sim* s) {
    size_t off = 0;
    for (auto& a : arrays) {
      CK(cudaMemcpyAsync(a.first, buf + off, a.second, cudaMemcpyDeviceToDevice, s->stream));
      off += a.second;
    }
    CK(cudaStreamSynchronize(s->stream));
  }
  ~TrialBackup() {
    if (buf) cudaFree(buf);
  }
};

template <class T>
void tune_group(ttsh_sim* s, Engine<T>& E, size_t gi, ttsh_tuning* out) {
  Group<T>& G = E.groups[gi];
  const int par = s->par;
  cudaStream_t st = s->stream;
  // launches per timed graph: more for small groups (a few microseconds per launch); the FFT
  // keeps 3 (repeated Poisson solves of one source grow by up to 1/k^2 each)
  const double sites = (double)G.N * G.N * G.N * G.n;
  const int reps = std::max(3, std::min(20, (int)(3e7 / sites)));
  const int reps_fft = 3;
  TrialBackup<T> bk;
  bk.save(s, E, gi);
  try {
    // the FFT, timed on a fresh Poisson source each time (the divergence launch refills W)
    auto fill = [&]() {
      if (s->fused) E.launch_fused_div_t(G, par, st);
      else launch_div<T>(G, par, st);
    };
    auto fft = [&]() {
      enqueue_fft(G, st, [](int, auto&& f) { f(); });
    };
    struct Cand { int kind, lb; std::vector<int> radix; };
    std::vector<Cand> cands;
    const std::vector<std::vector<int>> orders = radix_orders(G.N);
    if (fftreg_has<T>(G.N)) {
      cands.push_back({2, 0, orders[0]});
      cands.push_back({0, 0, orders[0]});
    }
    for (int lb : fft_lb_candidates<T>(G.N))
      for (const auto& o : orders) cands.push_back({1, lb, o});
    double best = 1e30;
    Cand pick = cands[0];
    for (const Cand& c : cands) {
      G.fft_kind = c.kind;
      G.fft_lb = c.lb;
      set_radix(s, E, gi, c.radix);
      const double t = time_graph(st, reps_fft, fill, fft);
      if (t < best) { best = t; pick = c; }
    }
    G.fft_kind = pick.kind;
    G.fft_lb = pick.lb;
    set_radix(s, E, gi, pick.radix);
    double ms[4] = {best, 0, 0, 0};
    if (s->fused) {
      // z-planes per CTA; 0: the persistent grid (equal shares of the group's sites per CTA)
      const int zcs[] = {0, 8, 16, 32, 64, 128, 256};
      for (int k = 0; k < 3; ++k) {
        double bk_t = 1e30;
        int bk_z = G.zc[k];
        for (int z : zcs) {
          if (z > G.N && z != zcs[1]) continue;
          if (z > 0 && (long)((G.N + z - 1) / z) * G.n > 65535) continue;
          G.zc[k] = z;
          const double t = time_graph(st, reps, [] {}, [&] {
            if (k == 0) E.launch_fused_rhs_t(G, par, st);
            else if (k == 1) E.launch_fused_div_t(G, par, st);
            else E.launch_fused_correct_t(G, par, st);
          });
          if (t < bk_t) { bk_t = t; bk_z = z; }
        }
        G.zc[k] = bk_z;
        ms[1 + k] = bk_t;
      }
    }
    bk.restore(s);
    for (int k = 0; k < 4; ++k) G.tuned_ms[k] = ms[k];
    get_tuning(s, E, gi, out);
  } catch (...) {
    try { bk.restore(s); } catch (...) {}
    throw;
  }
}

std::string tune_key(const ttsh_sim* s, int N, int n) {
  cudaDeviceProp pr{};
  CK(cudaGetDeviceProperties(&pr, s->device));
  std::string name = pr.name;
  for (char& c : name)
    if (c == ' ' || c == ':') c = '_';
  char buf[256];
  std::snprintf(buf, sizeof buf, "%s sm%d%d p%d f%d N%d n%d", name.c_str(), pr.major, pr.minor, s->precision,
                s->fused ? 1 : 0, N, n);
  return buf;
}

// Cache file: one line per entry, "<key> : kind lb zc0 zc1 zc2 nstages radix...".
std::map<std::string, ttsh_tuning> read_cache(const char* path) {
  std::map<std::string, ttsh_tuning> m;
  FILE* f = std::fopen(path, "r");
  if (!f) return m;
  char line[1024];
  while (std::fgets(line, sizeof line, f)) {
    const char* sep = std::strstr(line, " : ");
    if (!sep) continue;
    ttsh_tuning t{};
    int used = 0;
    if (std::sscanf(sep + 3, "%d %d %d %d %d %d%n", &t.fft_kind, &t.fft_lb, &t.zc[0], &t.zc[1], &t.zc[2],
                    &t.nstages, &used) != 6)
      continue;
    if (t.nstages < 1 || t.nstages > 16) continue;
    const char* q = sep + 3 + used;
    bool ok = true;
    for (int k = 0; k < t.nstages && ok; ++k) {
      int u = 0;
      ok = std::sscanf(q, "%d%n", &t.radix[k], &u) == 1;
      q += u;
    }
    if (ok) m[std::string(line, (size_t)(sep - line))] = t;
  }
  std::fclose(f);
  return m;
}

void append_cache(const char* path, const std::string& key, const ttsh_tuning& t) {
  FILE* f = std::fopen(path, "a");
  if (!f) throw std::runtime_error(std::string("tuning cache: cannot open ") + path);
  std::string line = key + " : " + std::to_string(t.fft_kind) + " " + std::to_string(t.fft_lb) + " " +
                     std::to_string(t.zc[0]) + " " + std::to_string(t.zc[1]) + " " + std::to_string(t.zc[2]) + " " +
                     std::to_string(t.nstages);
  for (int k = 0; k < t.nstages; ++k) line += " " + std::to_string(t.radix[k]);
  line += "\n";
  const bool ok = std::fputs(line.c_str(), f) >= 0;
  std::fclose(f);
  if (!ok) throw std::runtime_error(std::string("tuning cache: cannot write ") + path);
}

}  // namespace

// Whether kernels may read and write the host range [p, p + bytes) in place: it is page-locked
// (cudaHostAlloc / cudaHostRegister; in the unified address space its host address is also its
// device address), checked at both ends. Pageable arrays are staged by the copy engines.
static bool host_direct(const void* p, size_t bytes) {
  if (!p || !bytes) return false;
  const char* c = static_cast<const char*>(p);
  for (const char* q : {c, c + bytes - 1}) {
    cudaPointerAttributes at;
    if (cudaPointerGetAttributes(&at, q) != cudaSuccess) {
      (void)cudaGetLastError();
      return false;
    }
    if (at.type != cudaMemoryTypeHost || at.devicePointer != static_cast<const void*>(q)) return false;
  }
  return true;
}

// Host (FP64) <-> device (T) copies of one N^3 field, asynchronous on `st` (the caller
// synchronises). FP64 fields go through the copy engines. FP32 fields are converted on the device
// by kernels that read (write) the host array in place when host_direct allows it, and otherwise
// through `scratch`: n doubles of device memory that no step reads (the other half of the u*
// ping-pong pair, which the next step overwrites before reading); successive calls reuse it in
// stream order. scale_bits (FP32 only): see launch_to_f64.
template <class T>
static void h2d(ttsh_sim* s, T* dst, const double* src, size_t n, double* scratch) {
  const cudaStream_t st = s->stream;
  if constexpr (sizeof(T) == sizeof(double)) {
    CK(cudaMemcpyAsync(dst, src, n * sizeof(double), cudaMemcpyHostToDevice, st));
  } else {
    if (!host_direct(src, n * sizeof(double))) {
      CK(cudaMemcpyAsync(scratch, src, n * sizeof(double), cudaMemcpyHostToDevice, st));
      src = scratch;
    }
    launch_to_f32(src, dst, n, st);
  }
}
template <class T>
static void d2h(ttsh_sim* s, double* dst, const T* src, size_t n, double* scratch, size_t stride = 1,
                const int* scale_bits = nullptr) {
  const cudaStream_t st = s->stream;
  const bool direct = host_direct(dst, n * sizeof(double));
  if constexpr (sizeof(T) == sizeof(double)) {
    if (stride == 1) CK(cudaMemcpyAsync(dst, src, n * sizeof(double), cudaMemcpyDeviceToHost, st));
    else if (direct) launch_gather_f64(src, stride, dst, n, st);
    else CK(cudaMemcpy2DAsync(dst, sizeof(double), src, stride * sizeof(double), sizeof(double), n,
                              cudaMemcpyDeviceToHost, st));
  } else {
    launch_to_f64(src, stride, direct ? dst : scratch, n, scale_bits, st);
    if (!direct) CK(cudaMemcpyAsync(dst, scratch, n * sizeof(double), cudaMemcpyDeviceToHost, st));
  }
}
// The conversion scratch of an instance: its u* buffer of the parity not in use (three
// consecutive arena slots, >= 12 N^3 bytes), or nullptr for FP64 fields.
template <class I_>
static double* conv_scratch(const ttsh_sim* s, const I_& I) {
  typedef typename std::decay<decltype(*I.phi[0])>::type TT;
  if constexpr (std::is_same<TT, float>::value) {
    // fused: the pairs (u*, P*) of the parity not in use (24 N^3 bytes), which the next step rewrites
    if (I.star[0][0]) return reinterpret_cast<double*>(I.star[s->par ^ 1][0]);
    return reinterpret_cast<double*>(I.Us[s->par ^ 1][0]);
  } else {
    return nullptr;
  }
}

// The state arrays of a checkpoint, in file order, as (device pointer, bytes) of the current
// parity: phi, P, u of the element type, then u*, P* (the fused form: the (u*_b, P*_b) pairs, the
// phi compensation and the bf16 compensations of u and of the pairs): everything the next step
// reads.
template <class E>
static std::vector<std::pair<void*, size_t>> state_arrays(ttsh_sim* s, E& eng, int inst) {
  auto& I = eng.h[inst];
  typedef typename std::decay<decltype(*I.phi[0])>::type TT;
  const size_t n = (size_t)I.N * I.N * I.N, es = sizeof(TT), eb = sizeof(__nv_bfloat16);
  std::vector<std::pair<void*, size_t>> a = {{I.phi[s->par], n * es}};
  for (int b = 0; b < 3; ++b) a.push_back({I.P[b], n * es});
  for (int b = 0; b < 3; ++b) a.push_back({I.U[b], n * es});
  if (I.phic) {  // fused: the pairs (u*_b, P*_b) and their compensations
    for (int b = 0; b < 3; ++b) a.push_back({I.star[s->par][b], 2 * n * es});
    a.push_back({I.phic, n * es});
    for (int f = 0; f < 3; ++f) a.push_back({I.lo[f], n * eb});
    for (int b = 0; b < 3; ++b) a.push_back({I.starlo[s->par][b], 2 * n * eb});
    return a;
  }
  for (int b = 0; b < 3; ++b) a.push_back({I.Us[s->par][b], n * es});
  for (int b = 0; b < 3; ++b) a.push_back({I.Ps[s->par][b], n * es});
  return a;
}

// Host-side reduction of one group's diagnostics partials (per droplet: blocks x {sum, max|D.u|,
// max|u|, non-finite count}, fixed order) into ttsh_stats; returns whether any value is non-finite.
template <class E>
static bool stats_of_group(const ttsh_sim* s, const E& eng, size_t g, int what, const double* part, int64_t steps,
                           const double* T, ttsh_stats* out) {
  const size_t per = 4 * (size_t)stats_partials_per_instance(0);
  bool bad_any = false;
  for (size_t k = 0; k < eng.members[g].size(); ++k) {
    const int inst = eng.members[g][k];
    double sum = 0, md = 0, mu = 0, bad = 0;
    for (size_t b = 0; b < per / 4; ++b) {
      const double* q = &part[k * per + 4 * b];
      sum += q[0];
      md = std::max(md, q[1]);
      mu = std::max(mu, q[2]);
      bad += q[3];
    }
    const double h = s->inst[inst].in.h;
    ttsh_stats& o = out[inst];
    o.mass = sum * h * h * h;
    o.max_div_u = what == TTSH_STATS_ALL ? md : -1.0;
    o.max_abs_u = what == TTSH_STATS_ALL ? mu : -1.0;
    o.T = T[inst];
    o.steps = steps;
    o.nonfinite = bad > 0 ? 1 : 0;
    o.reserved = 0;
    if (bad > 0) bad_any = true;
  }
  return bad_any;
}

extern "C" {

int ttsh_batch_create(const ttsh_input* in, const ttsh_ext* ext, int n, int device, ttsh_sim** out) {
  if (!in || !out || n <= 0) return set_error(TTSH_E_INVALID, "ttsh_batch_create: bad arguments");
  *out = nullptr;
  ttsh_ext dflt;
  ttsh_default_ext(&dflt);
  for (int i = 0; i < n; ++i) {
    int rc = validate(in[i], ext ? ext[i] : dflt);
    if (rc) return rc;
    if ((ext ? ext[i].precision : dflt.precision) != (ext ? ext[0].precision : dflt.precision))
      return set_error(TTSH_E_INVALID, "all instances of a batch share one precision");
    if ((ext ? ext[i].form : dflt.form) != (ext ? ext[0].form : dflt.form))
      return set_error(TTSH_E_INVALID, "all instances of a batch share one form");
  }
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    return set_error(TTSH_E_NODEVICE, "no CUDA device visible (check CUDA_VISIBLE_DEVICES)");
  }
  ttsh_sim* s = new ttsh_sim();
  return guarded([&]() -> int {
    try {
      if (device < 0) CK(cudaGetDevice(&device));
      if (device >= ndev) throw std::runtime_error("device index out of range");
      s->device = device;
      CK(cudaSetDevice(device));
      CK(cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking));
      s->own_stream = true;
      s->precision = ext ? ext[0].precision : dflt.precision;
      s->inst.resize(n);
      for (int i = 0; i < n; ++i) {
        s->inst[i].in = in[i];
        s->inst[i].ext = ext ? ext[i] : dflt;
        s->inst[i].N = in[i].Nx;
        s->inst[i].T = in[i].T0;
      }
      const int form = pick_form(s);
      if (form < 0) {
        release(s);
        s = nullptr;
        return set_error(TTSH_E_UNSUPPORTED, "fused form needs FP32 and N a multiple of 32");
      }
      s->fused = form == 1;
      if (s->fused) fused_prepare();
      if (s->precision == 32) build_engine<float>(s, s->ef);
      else build_engine<double>(s, s->ed);
      capture_graphs(s);
      CK(cudaStreamSynchronize(s->stream));
      *out = s;
      return TTSH_OK;
    } catch (...) {
      release(s);
      throw;
    }
  });
}

int ttsh_create(const ttsh_input* in, const ttsh_ext* ext, int device, ttsh_sim** out) {
  return ttsh_batch_create(in, ext, 1, device, out);
}

int ttsh_set_stream(ttsh_sim* s, void* stream) {
  if (!s) return set_error(TTSH_E_INVALID, "null handle");
  return guarded([&]() -> int {
    CK(cudaSetDevice(s->device));
    CK(cudaStreamSynchronize(s->stream));
    if (stream) {
      if (s->own_stream) CK(cudaStreamDestroy(s->stream));
      s->own_stream = false;
      s->stream = (cudaStream_t)stream;
    } else if (!s->own_stream) {
      CK(cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking));
      s->own_stream = true;
    }
    return TTSH_OK;
  });
}

void ttsh_destroy(ttsh_sim* s) { release(s); }

int ttsh_num_instances(const ttsh_sim* s) { return s ? (int)s->inst.size() : 0; }
int ttsh_instance_n(const ttsh_sim* s, int inst) {
  return (s && inst >= 0 && inst < (int)s->inst.size()) ? s->inst[inst].N : 0;
}
double ttsh_time(const ttsh_sim* s) { return (s && !s->inst.empty()) ? s->inst[0].T : 0.0; }
int ttsh_launches_per_step(const ttsh_sim* s) {
  if (!s) return 0;
  return s->precision == 32 ? s->ef.launches(s->fused) : s->ed.launches(s->fused);
}

static int check_inst(ttsh_sim* s, int inst) {
  if (!s) return set_error(TTSH_E_INVALID, "null handle");
  if (inst < 0 || inst >= (int)s->inst.size()) return set_error(TTSH_E_INVALID, "instance index out of range");
  return TTSH_OK;
}

int ttsh_set_state(ttsh_sim* s, int inst, const double* phi, const double* P, const double* u, const double* ustar,
                   const double* Pstar) {
  int rc = check_inst(s, inst);
  if (rc) return rc;
  if (!phi || !P || !u) return set_error(TTSH_E_INVALID, "phi, P and u are required");
  return guarded([&]() -> int {
    CK(cudaSetDevice(s->device));
    CK(cudaStreamSynchronize(s->stream));
    const int N = s->inst[inst].N;
    const size_t n = (size_t)N * N * N;
    if (s->fused) {
      // compensated fields: FP32 value + remainder; no grid for the first divergence yet
      InstDev<float>& I = s->ef.h[inst];
      double* scr = conv_scratch(s, I);
      // the split kernel reads the host array in place when it can (host_direct), else a staged copy
      auto stage = [&](const double* src) -> const double* {
        if (host_direct(src, n * sizeof(double))) return src;
        CK(cudaMemcpyAsync(scr, src, n * sizeof(double), cudaMemcpyHostToDevice, s->stream));
        return scr;
      };
      auto put = [&](const double* src, float* hi, __nv_bfloat16* lo, float* lo32) {
        launch_split(stage(src), hi, lo, lo32, n, 1, s->stream);
      };
      auto put2 = [&](const double* src, float* hi, __nv_bfloat16* lo) {  // one half of the pairs
        launch_split(stage(src), hi, lo, nullptr, n, 2, s->stream);
      };
      put(phi, I.phi[s->par], nullptr, I.phic);
      for (int b = 0; b < 3; ++b) {
        put(u + b * n, I.U[b], I.lo[b], nullptr);
        put(P + b * n, I.P[b], nullptr, nullptr);
        // the previous u*, P* (the stale halo of the first divergence) into the pairs' halves
        float* sh = reinterpret_cast<float*>(I.star[s->par][b]);
        __nv_bfloat16* sl = reinterpret_cast<__nv_bfloat16*>(I.starlo[s->par][b]);
        if (!ustar || !Pstar) {
          CK(cudaMemsetAsync(sh, 0, 2 * n * sizeof(float), s->stream));
          CK(cudaMemsetAsync(sl, 0, 2 * n * sizeof(__nv_bfloat16), s->stream));
        }
        if (ustar) put2(ustar + b * n, sh, sl);
        if (Pstar) put2(Pstar + b * n, sh + 1, sl + 1);
      }
      CK(cudaMemsetAsync(I.smax, 0, 2 * sizeof(int), s->stream));
      CK(cudaStreamSynchronize(s->stream));
      return TTSH_OK;
    }
    s->with_engine([&](auto& E) {
      auto& I = E.h[inst];
      typedef typename std::decay<decltype(*I.phi[0])>::type TT;
      double* scr = conv_scratch(s, I);
      h2d<TT>(s, I.phi[s->par], phi, n, scr);
      if (I.phic) CK(cudaMemsetAsync(I.phic, 0, n * sizeof(TT), s->stream));
      for (int b = 0; b < 3; ++b) {
        h2d<TT>(s, I.P[b], P + b * n, n, scr);
        h2d<TT>(s, I.U[b], u + b * n, n, scr);
        if (ustar) h2d<TT>(s, I.Us[s->par][b], ustar + b * n, n, scr);
        else CK(cudaMemsetAsync(I.Us[s->par][b], 0, n * sizeof(TT), s->stream));
        if (Pstar) h2d<TT>(s, I.Ps[s->par][b], Pstar + b * n, n, scr);
        else CK(cudaMemsetAsync(I.Ps[s->par][b], 0, n * sizeof(TT), s->stream));
      }
      CK(cudaStreamSynchronize(s->stream));
    });
    return TTSH_OK;
  });
}

int ttsh_step(ttsh_sim* s, int nsteps) {
  if (!s || nsteps < 0) return set_error(TTSH_E_INVALID, "ttsh_step: bad arguments");
  return guarded([&]() -> int {
    CK(cudaSetDevice(s->device));
    for (int t = 0; t < nsteps; ++t) {
      CK(cudaGraphLaunch(s->gexec[s->par], s->stream));
      s->par ^= 1;
      s->steps += 1;
      for (auto& ih : s->inst) ih.T = ih.T + ih.in.dt0;  // run(): T = T + Dt (TTSH3D.cu:342)
    }
    return TTSH_OK;
  });
}

int ttsh_sync(ttsh_sim* s) {
  if (!s) return set_error(TTSH_E_INVALID, "null handle");
  return guarded([&]() -> int {
    CK(cudaSetDevice(s->device));
    CK(cudaStreamSynchronize(s->stream));
    return kernel_error(s);
  });
}

int ttsh_get_state(ttsh_sim* s, int inst, double* phi, double* P, double* u, double* p_v, double* p_p) {
  int rc = check_inst(s, inst);
  if (rc) return rc;
  return guarded([&]() -> int {
    CK(cudaSetDevice(s->device));
    CK(cudaStreamSynchronize(s->stream));
    const int N = s->inst[inst].N;
    const size_t n = (size_t)N * N * N;
    s->with_engine([&](auto& E) {
      auto& I = E.h[inst];
      typedef typename std::decay<decltype(*I.phi[0])>::type TT;
      double* scr = conv_scratch(s, I);
      if constexpr (std::is_same<TT, float>::value) {
        if (s->fused) {  // the compensated values
          auto get = [&](double* dst, const float* hi, const __nv_bfloat16* lo, const float* lo32) {
            if (host_direct(dst, n * sizeof(double))) {  // joined straight into the host array
              launch_join(hi, lo, lo32, dst, n, 1, s->stream);
              return;
            }
            launch_join(hi, lo, lo32, scr, n, 1, s->stream);
            CK(cudaMemcpyAsync(dst, scr, n * sizeof(double), cudaMemcpyDeviceToHost, s->stream));
          };
          if (phi) get(phi, I.phi[s->par], nullptr, I.phic);
          for (int b = 0; b < 3; ++b) {
            if (P) get(P + b * n, I.P[b], nullptr, nullptr);
            if (u) get(u + b * n, I.U[b], I.lo[b], nullptr);
          }
        }
      }
      if (!s->fused) {
        if (phi) d2h<TT>(s, phi, I.phi[s->par], n, scr);
        for (int b = 0; b < 3; ++b) {
          if (P) d2h<TT>(s, P + b * n, I.P[b], n, scr);
          if (u) d2h<TT>(s, u + b * n, I.U[b], n, scr);
        }
      }
      // FP32: the pressures come out of the FFT scaled by powers of two (pow2_norm, common.cuh),
      // recorded as the maxima wmax[0], wmax[1]; FP64: unscaled (wmax is null)
      const TT* w = reinterpret_cast<const TT*>(I.W);
      const int* wm = I.wmax;
      if (p_v) d2h<TT>(s, p_v, w, n, scr, 2, wm);
      if (p_p) d2h<TT>(s, p_p, w + 1, n, scr, 2, wm ? wm + 1 : nullptr);
      CK(cudaStreamSynchronize(s->stream));
    });
    return kernel_error(s);
  });
}

int ttsh_get_provisional(ttsh_sim* s, int inst, double* ustar, double* Pstar) {
  int rc = check_inst(s, inst);
  if (rc) return rc;
  return guarded([&]() -> int {
    CK(cudaSetDevice(s->device));
    CK(cudaStreamSynchronize(s->stream));
    const int N = s->inst[inst].N;
    const size_t n = (size_t)N * N * N;
    s->with_engine([&](auto& E) {
      auto& I = E.h[inst];
      typedef typename std::decay<decltype(*I.phi[0])>::type TT;
      double* scr = conv_scratch(s, I);
      for (int b = 0; b < 3; ++b) {
        if constexpr (std::is_same<TT, float>::value) {
          if (s->fused) {  // the last step's u*, P*, compensated (the halves of the pairs)
            const float* sh = reinterpret_cast<const float*>(I.star[s->par][b]);
            const __nv_bfloat16* sl = reinterpret_cast<const __nv_bfloat16*>(I.starlo[s->par][b]);
            auto get2 = [&](double* dst, const float* hi, const __nv_bfloat16* lo) {  // one half of the pairs
              if (host_direct(dst, n * sizeof(double))) {
                launch_join(hi, lo, nullptr, dst, n, 2, s->stream);
                return;
              }
              launch_join(hi, lo, nullptr, scr, n, 2, s->stream);
              CK(cudaMemcpyAsync(dst, scr, n * sizeof(double), cudaMemcpyDeviceToHost, s->stream));
            };
            if (ustar) get2(ustar + b * n, sh, sl);
            if (Pstar) get2(Pstar + b * n, sh + 1, sl + 1);
            continue;
          }
        }
        if (ustar) d2h<TT>(s, ustar + b * n, I.Us[s->par][b], n, scr);
        if (Pstar) d2h<TT>(s, Pstar + b * n, I.Ps[s->par][b], n, scr);
      }
      CK(cudaStreamSynchronize(s->stream));
    });
    return TTSH_OK;
  });
}

int ttsh_reduce(ttsh_sim* s, int inst, ttsh_stats* out) {
  int rc = check_inst(s, inst);
  if (rc) return rc;
  if (!out) return set_error(TTSH_E_INVALID, "null stats");
  return guarded([&]() -> int {
    CK(cudaSetDevice(s->device));
    const InstHost& ih = s->inst[inst];
    std::vector<double> part;
    s->with_engine([&](auto& E) {
      const int g = E.grp[inst];
      const int nb = launch_stats(E.groups[g], s->par, s->stream);
      part.resize(4 * (size_t)nb);
      CK(cudaMemcpyAsync(part.data(), E.h[inst].red, part.size() * sizeof(double), cudaMemcpyDeviceToHost,
                         s->stream));
      CK(cudaStreamSynchronize(s->stream));
    });
    double sum = 0, md = 0, mu = 0, bad = 0;
    for (size_t b = 0; b < part.size() / 4; ++b) {
      sum += part[4 * b];
      md = std::max(md, part[4 * b + 1]);
      mu = std::max(mu, part[4 * b + 2]);
      bad += part[4 * b + 3];
    }
    const double h = ih.in.h;
    out->mass = sum * h * h * h;
    out->max_div_u = md;
    out->max_abs_u = mu;
    out->T = ih.T;
    out->steps = s->steps;
    out->nonfinite = bad > 0 ? 1 : 0;
    out->reserved = 0;
    return bad > 0 ? set_error(TTSH_E_UNSTABLE, "non-finite values in the state") : TTSH_OK;
  });
}

int ttsh_reduce_all(ttsh_sim* s, int what, ttsh_stats* out) {
  if (!s || !out) return set_error(TTSH_E_INVALID, "null argument");
  if (what != TTSH_STATS_ALL && what != TTSH_STATS_MASS) return set_error(TTSH_E_INVALID, "bad stats selector");
  return guarded([&]() -> int {
    CK(cudaSetDevice(s->device));
    bool bad_any = false;
    std::vector<double> T(s->inst.size());
    for (size_t i = 0; i < T.size(); ++i) T[i] = s->inst[i].T;
    s->with_engine([&](auto& E) {
      const size_t per = 4 * (size_t)stats_partials_per_instance(0);
      for (size_t g = 0; g < E.groups.size(); ++g) {
        const auto& G = E.groups[g];
        launch_stats(G, s->par, s->stream, what == TTSH_STATS_ALL);
        std::vector<double> part(per * G.n);
        CK(cudaMemcpyAsync(part.data(), G.red, part.size() * sizeof(double), cudaMemcpyDeviceToHost, s->stream));
        CK(cudaStreamSynchronize(s->stream));
        if (stats_of_group(s, E, g, what, part.data(), s->steps, T.data(), out)) bad_any = true;
      }
    });
    return bad_any ? set_error(TTSH_E_UNSTABLE, "non-finite values in the state") : TTSH_OK;
  });
}

// Layout of an asynchronous diagnostics buffer: [steps, what, T of each droplet, then the
// partials of every group in group order].
static size_t partials_doubles(const ttsh_sim* s) {
  size_t n = 2 + s->inst.size();
  const size_t per = 4 * (size_t)stats_partials_per_instance(0);
  return n + per * s->inst.size();
}

size_t ttsh_partials_size(const ttsh_sim* s) { return s ? partials_doubles(s) : 0; }

int ttsh_reduce_all_async(ttsh_sim* s, int what, double* partials) {
  if (!s || !partials) return set_error(TTSH_E_INVALID, "null argument");
  if (what != TTSH_STATS_ALL && what != TTSH_STATS_MASS) return set_error(TTSH_E_INVALID, "bad stats selector");
  return guarded([&]() -> int {
    CK(cudaSetDevice(s->device));
    partials[0] = (double)s->steps;
    partials[1] = (double)what;
    for (size_t i = 0; i < s->inst.size(); ++i) partials[2 + i] = s->inst[i].T;
    double* dst = partials + 2 + s->inst.size();
    s->with_engine([&](auto& E) {
      const size_t per = 4 * (size_t)stats_partials_per_instance(0);
      for (size_t g = 0; g < E.groups.size(); ++g) {
        const auto& G = E.groups[g];
        launch_stats(G, s->par, s->stream, what == TTSH_STATS_ALL);
        CK(cudaMemcpyAsync(dst, G.red, per * G.n * sizeof(double), cudaMemcpyDeviceToHost, s->stream));
        dst += per * G.n;
      }
    });
    return TTSH_OK;
  });
}

int ttsh_stats_from_partials(const ttsh_sim* s, const double* partials, ttsh_stats* out) {
  if (!s || !partials || !out) return set_error(TTSH_E_INVALID, "null argument");
  const int what = (int)partials[1];
  if (what != TTSH_STATS_ALL && what != TTSH_STATS_MASS) return set_error(TTSH_E_INVALID, "not a diagnostics buffer");
  bool bad_any = false;
  const double* T = partials + 2;
  const double* part = partials + 2 + s->inst.size();
  const size_t per = 4 * (size_t)stats_partials_per_instance(0);
  auto run = [&](const auto& E) {
    for (size_t g = 0; g < E.groups.size(); ++g) {
      if (stats_of_group(s, E, g, what, part, (int64_t)partials[0], T, out)) bad_any = true;
      part += per * E.groups[g].n;
    }
  };
  if (s->precision == 32) run(s->ef);
  else run(s->ed);
  return bad_any ? set_error(TTSH_E_UNSTABLE, "non-finite values in the state") : TTSH_OK;
}

// Waits for the snapshot the writer thread is formatting; its status (and message) becomes the
// caller's.
static int conf_join(ttsh_sim* s) {
  if (!s->conf_thread.joinable()) return TTSH_OK;
  s->conf_thread.join();
  const int rc = s->conf_rc;
  s->conf_rc = 0;
  return rc ? set_error(rc, s->conf_msg) : TTSH_OK;
}

int ttsh_write_conf_async(ttsh_sim* s, int inst, const char* path) {
  int rc = check_inst(s, inst);
  if (rc) return rc;
  if (!path) return set_error(TTSH_E_INVALID, "null path");
  rc = conf_join(s);  // one buffer: the previous snapshot is finished first
  if (rc) return rc;
  return guarded([&]() -> int {
    CK(cudaSetDevice(s->device));
    const int N = s->inst[inst].N;
    const size_t n = (size_t)N * N * N;
    if (s->conf_cap < 7 * n) {
      CK(cudaStreamSynchronize(s->stream));
      if (s->conf_buf) CK(cudaFreeHost(s->conf_buf));
      s->conf_buf = nullptr;
      s->conf_cap = 0;
      CK(cudaHostAlloc(&s->conf_buf, 7 * n * sizeof(double), cudaHostAllocDefault));
      s->conf_cap = 7 * n;
    }
    if (!s->conf_ready) CK(cudaEventCreateWithFlags(&s->conf_ready, cudaEventDisableTiming));
    double* u = s->conf_buf;
    double* P = u + 3 * n;
    double* phi = P + 3 * n;
    // the device writes the FP64 values straight into the page-locked buffer (it is mapped in the
    // unified address space), in stream order: later steps may be enqueued right away
    s->with_engine([&](auto& E) {
      auto& I = E.h[inst];
      typedef typename std::decay<decltype(*I.phi[0])>::type TT;
      if constexpr (std::is_same<TT, float>::value) {
        if (s->fused) {
          launch_join(I.phi[s->par], nullptr, I.phic, phi, n, 1, s->stream);
          for (int b = 0; b < 3; ++b) {
            launch_join(I.U[b], I.lo[b], nullptr, u + b * n, n, 1, s->stream);
            launch_join(I.P[b], nullptr, nullptr, P + b * n, n, 1, s->stream);
          }
        } else {
          launch_to_f64(I.phi[s->par], 1, phi, n, nullptr, s->stream);
          for (int b = 0; b < 3; ++b) {
            launch_to_f64(I.U[b], 1, u + b * n, n, nullptr, s->stream);
            launch_to_f64(I.P[b], 1, P + b * n, n, nullptr, s->stream);
          }
        }
      } else {
        CK(cudaMemcpyAsync(phi, I.phi[s->par], n * sizeof(double), cudaMemcpyDeviceToHost, s->stream));
        for (int b = 0; b < 3; ++b) {
          CK(cudaMemcpyAsync(u + b * n, I.U[b], n * sizeof(double), cudaMemcpyDeviceToHost, s->stream));
          CK(cudaMemcpyAsync(P + b * n, I.P[b], n * sizeof(double), cudaMemcpyDeviceToHost, s->stream));
        }
      }
    });
    CK(cudaEventRecord(s->conf_ready, s->stream));
    const int expo = s->inst[inst].in.ExpoData, dev = s->device;
    const std::string file = path;
    cudaEvent_t ev = s->conf_ready;
    s->conf_thread = std::thread([s, N, expo, dev, file, ev, u, P, phi]() {
      cudaSetDevice(dev);
      const cudaError_t e = cudaEventSynchronize(ev);
      if (e != cudaSuccess) {
        s->conf_rc = TTSH_E_CUDA;
        s->conf_msg = std::string("snapshot copy: ") + cudaGetErrorString(e);
        return;
      }
      s->conf_rc = ttsh_format_conf(N, expo, phi, P, u, file.c_str());
      if (s->conf_rc) s->conf_msg = ttsh_last_error();
    });
    return TTSH_OK;
  });
}

int ttsh_conf_wait(ttsh_sim* s) {
  if (!s) return set_error(TTSH_E_INVALID, "null handle");
  return conf_join(s);
}

int ttsh_write_conf(ttsh_sim* s, int inst, const char* path) {
  int rc = ttsh_write_conf_async(s, inst, path);
  return rc ? rc : conf_join(s);
}

int ttsh_snapshot_slice(ttsh_sim* s, int inst, double* centroid, int* index, double* slices) {
  int rc = check_inst(s, inst);
  if (rc) return rc;
  return guarded([&]() -> int {
    CK(cudaSetDevice(s->device));
    const int N = s->inst[inst].N;
    const size_t NN = (size_t)N * N;
    const size_t need = (9 * NN + 4 * (size_t)centroid_blocks()) * sizeof(double);
    if (s->post_bytes < need) {
      CK(cudaStreamSynchronize(s->stream));
      if (s->post) CK(cudaFree(s->post));
      s->post = nullptr;
      CK(cudaMalloc(&s->post, need));
      s->post_bytes = need;
    }
    double* part = s->post + 9 * NN;
    std::vector<double> hp(4 * (size_t)centroid_blocks());
    double c[3];
    int idx[3];
    s->with_engine([&](auto& E) {
      const auto& g = E.groups[E.grp[inst]];
      launch_centroid(g.d_inst, E.loc[inst], s->par, part, s->stream);
      CK(cudaMemcpyAsync(hp.data(), part, hp.size() * sizeof(double), cudaMemcpyDeviceToHost, s->stream));
      CK(cudaStreamSynchronize(s->stream));
      double a[4] = {0, 0, 0, 0};
      for (size_t b = 0; b < hp.size() / 4; ++b)
        for (int q = 0; q < 4; ++q) a[q] += hp[4 * b + q];
      for (int q = 0; q < 3; ++q) {
        c[q] = a[q + 1] / a[0];
        idx[q] = (int)c[q];  // Python int(): truncation toward zero
      }
      if (slices) {
        const int zs = ((idx[2] % N) + N) % N;
        launch_slice(g.d_inst, E.loc[inst], s->par, N, zs, s->post, s->stream);
        CK(cudaMemcpyAsync(slices, s->post, 9 * NN * sizeof(double), cudaMemcpyDeviceToHost, s->stream));
        CK(cudaStreamSynchronize(s->stream));
      }
    });
    for (int q = 0; q < 3; ++q) {
      if (centroid) centroid[q] = c[q];
      if (index) index[q] = idx[q];
    }
    return TTSH_OK;
  });
}

int ttsh_run_dirs(const char* const* dirs, int n, const ttsh_ext* ext, uint64_t seed, int device) {
  if (!dirs || n <= 0) return set_error(TTSH_E_INVALID, "ttsh_run_dirs: bad arguments");
  std::vector<ttsh_input> in(n);
  std::vector<ttsh_ext> ex(n);
  ttsh_ext d;
  ttsh_default_ext(&d);
  for (int i = 0; i < n; ++i) {
    int rc = ttsh_read_input((std::string(dirs[i]) + "/input.dat").c_str(), &in[i]);
    if (rc) return rc;
    ex[i] = ext ? *ext : d;
  }
  ttsh_sim* s = nullptr;
  int rc = ttsh_batch_create(in.data(), ex.data(), n, device, &s);
  if (rc) return rc;
  struct Run {
    double T, Dt, dte, Ts;
    bool active;
  };
  std::vector<Run> run(n);
  // The initial states (the reference's generator, sequential within a droplet) are computed for
  // several droplets at once on host threads, as many as fit in about 4 GiB of host arrays (13 N^3
  // doubles each), then uploaded and written in directory order.
  struct Init {
    std::vector<double> phi, P, u, us, Ps;
    int rc = 0;
    std::string msg;
  };
  size_t per = 0;
  for (int i = 0; i < n; ++i) per = std::max(per, 13 * (size_t)in[i].Nx * in[i].Nx * in[i].Nx * sizeof(double));
  const int conc = (int)std::max<size_t>(
      1, std::min<size_t>(std::max(1u, std::thread::hardware_concurrency()), ((size_t)4 << 30) / std::max<size_t>(per, 1)));
  for (int b = 0; b < n; b += conc) {
    const int e = std::min(n, b + conc);
    std::vector<Init> ini(e - b);
    std::vector<std::thread> th;
    for (int i = b; i < e; ++i)
      th.emplace_back([&, i]() {
        const ttsh_input& p = in[i];
        const size_t nn = (size_t)p.Nx * p.Nx * p.Nx;
        Init& w = ini[i - b];
        w.phi.resize(nn);
        w.P.resize(3 * nn);
        w.u.resize(3 * nn);
        w.us.resize(3 * nn);
        w.Ps.resize(3 * nn);
        const int t0 = (int)((p.T0 + 0.1 * p.dte) / p.dte);  // TTSH3D.cu:768
        const std::string conf0 = std::string(dirs[i]) + "/../data/conf_" + std::to_string(t0) + ".dat";
        w.rc = ttsh_init_reference(&p, (unsigned)(seed + (uint64_t)i), conf0.c_str(), w.phi.data(), w.P.data(),
                                   w.u.data(), w.us.data(), w.Ps.data());
        if (w.rc) w.msg = ttsh_last_error();  // the error text is per thread
      });
    for (auto& t : th) t.join();
    for (int i = b; i < e && !rc; ++i) {
      const ttsh_input& p = in[i];
      Init& w = ini[i - b];
      rc = w.rc ? set_error(w.rc, w.msg) : 0;
      if (!rc) rc = ttsh_set_state(s, i, w.phi.data(), w.P.data(), w.u.data(), w.us.data(), w.Ps.data());
      if (!rc && p.T0 == 0) rc = ttsh_write_conf(s, i, (std::string(dirs[i]) + "/conf_0.dat").c_str());
      run[i] = {p.T0, p.dt0, p.dte, p.Ts, true};
    }
    if (rc) {
      ttsh_destroy(s);
      return rc;
    }
  }
  // opt-in autotuning (TTSH_TUNE=1; TTSH_TUNE_CACHE names a cache file), on the initial fields
  if (const char* tv = std::getenv("TTSH_TUNE")) {
    if (std::atoi(tv) != 0) {
      int rt = ttsh_autotune(s, std::getenv("TTSH_TUNE_CACHE"));
      if (rt) {
        ttsh_destroy(s);
        return rt;
      }
    }
  }
  // evolve() of every droplet in lockstep (TTSH3D.cu:311-331): advance to the nearest event
  for (;;) {
    int nact = 0;
    int k = 1 << 30;
    for (int i = 0; i < n; ++i) {
      if (!run[i].active) continue;
      ++nact;
      double T = run[i].T;
      int m = 0;
      for (;;) {  // steps until this droplet's next snapshot or stop
        T = T + run[i].Dt;
        ++m;
        if (std::floor(T / run[i].dte) > std::floor((T - run[i].Dt) / run[i].dte) || T > run[i].Ts || m >= (1 << 20))
          break;
      }
      k = std::min(k, m);
    }
    if (nact == 0) break;
    if ((rc = ttsh_step(s, k)) != 0) break;
    for (int i = 0; i < n && !rc; ++i) {
      if (!run[i].active) {
        for (int m = 0; m < k; ++m) run[i].T = run[i].T + run[i].Dt;
        continue;
      }
      for (int m = 0; m < k && !rc; ++m) {
        run[i].T = run[i].T + run[i].Dt;
        if (m + 1 < k) continue;  // events only happen at the k-th step (k is the minimum distance)
        if (std::floor(run[i].T / run[i].dte) > std::floor((run[i].T - run[i].Dt) / run[i].dte)) {
          const long te = (long)std::floor(run[i].T / run[i].dte);
          // formatted while the next steps run
          rc = ttsh_write_conf_async(s, i, (std::string(dirs[i]) + "/conf_" + std::to_string(te) + ".dat").c_str());
        }
        if (run[i].T > run[i].Ts) run[i].active = false;
      }
    }
    if (rc) break;
  }
  const int wrc = ttsh_conf_wait(s);
  ttsh_destroy(s);
  return rc ? rc : wrc;
}

static const char kCkpMagic[8] = {'T', 'T', 'S', 'H', 'C', 'K', 'P', '1'};

// Checkpoint file: "TTSHCKP1", int32 {1, N, precision, arrays beyond the first 13}, FP64 T, int64
// steps, then the state arrays (state_arrays) as raw device bytes.
int ttsh_save_checkpoint(ttsh_sim* s, int inst, const char* path) {
  int rc = check_inst(s, inst);
  if (rc) return rc;
  if (!path) return set_error(TTSH_E_INVALID, "null path");
  return guarded([&]() -> int {
    CK(cudaSetDevice(s->device));
    CK(cudaStreamSynchronize(s->stream));
    const int N = s->inst[inst].N;
    FILE* fp = std::fopen(path, "wb");
    if (!fp) return set_error(TTSH_E_IO, std::string("cannot open ") + path);
    std::vector<std::pair<void*, size_t>> arr;
    s->with_engine([&](auto& E) { arr = state_arrays(s, E, inst); });
    int32_t hdr[4] = {1, N, s->precision, (int32_t)arr.size() - 13};
    double T = s->inst[inst].T;
    int64_t steps = s->steps;
    bool ok = std::fwrite(kCkpMagic, 1, 8, fp) == 8 && std::fwrite(hdr, 4, 4, fp) == 4 &&
              std::fwrite(&T, 8, 1, fp) == 1 && std::fwrite(&steps, 8, 1, fp) == 1;
    std::vector<char> buf;
    for (const auto& a : arr) {
      if (!ok) break;
      buf.resize(a.second);
      CK(cudaMemcpy(buf.data(), a.first, a.second, cudaMemcpyDeviceToHost));
      ok = std::fwrite(buf.data(), 1, a.second, fp) == a.second;
    }
    if (std::fclose(fp) != 0) ok = false;
    return ok ? TTSH_OK : set_error(TTSH_E_IO, std::string("write failed: ") + path);
  });
}

int ttsh_load_checkpoint(ttsh_sim* s, int inst, const char* path) {
  int rc = check_inst(s, inst);
  if (rc) return rc;
  if (!path) return set_error(TTSH_E_INVALID, "null path");
  return guarded([&]() -> int {
    CK(cudaSetDevice(s->device));
    CK(cudaStreamSynchronize(s->stream));
    const int N = s->inst[inst].N;
    FILE* fp = std::fopen(path, "rb");
    if (!fp) return set_error(TTSH_E_IO, std::string("cannot open ") + path);
    char magic[8];
    int32_t hdr[4];
    double T;
    int64_t steps;
    bool ok = std::fread(magic, 1, 8, fp) == 8 && std::memcmp(magic, kCkpMagic, 8) == 0 &&
              std::fread(hdr, 4, 4, fp) == 4 && std::fread(&T, 8, 1, fp) == 1 && std::fread(&steps, 8, 1, fp) == 1;
    if (!ok || hdr[0] != 1) {
      std::fclose(fp);
      return set_error(TTSH_E_PARSE, std::string("not a ttsh checkpoint: ") + path);
    }
    std::vector<std::pair<void*, size_t>> arr;
    s->with_engine([&](auto& E) { arr = state_arrays(s, E, inst); });
    if (hdr[1] != N || hdr[2] != s->precision || hdr[3] != (int32_t)arr.size() - 13) {
      std::fclose(fp);
      return set_error(TTSH_E_INVALID, "checkpoint size, precision or form differs from the instance");
    }
    std::vector<char> buf;
    for (const auto& a : arr) {
      buf.resize(a.second);
      if (std::fread(buf.data(), 1, a.second, fp) != a.second) {
        std::fclose(fp);
        return set_error(TTSH_E_PARSE, std::string("truncated checkpoint: ") + path);
      }
      CK(cudaMemcpy(a.first, buf.data(), a.second, cudaMemcpyHostToDevice));
    }
    std::fclose(fp);
    s->inst[inst].T = T;
    return TTSH_OK;
  });
}

int ttsh_profile_kernels(ttsh_sim* s, int nsteps, int cap, const char** names, double* ms_per_step,
                         int64_t* launches_per_step) {
  if (!s || nsteps <= 0 || cap <= 0 || !names || !ms_per_step) return set_error(TTSH_E_INVALID, "bad arguments");
  int written = 0;
  int rc = guarded([&]() -> int {
    CK(cudaSetDevice(s->device));
    Prof pr;
    pr.st = s->stream;
    for (int t = 0; t < nsteps; ++t) {
      s->with_engine([&](auto& E) { E.enqueue_step(s->par, s->stream, s->fused, &pr); });
      s->par ^= 1;
      s->steps += 1;
      for (auto& ih : s->inst) ih.T = ih.T + ih.in.dt0;
    }
    CK(cudaStreamSynchronize(s->stream));
    std::vector<double> tot(K_NCLASS, 0.0);
    std::vector<int64_t> cnt(K_NCLASS, 0);
    for (auto& e : pr.ev) {
      float ms = 0;
      CK(cudaEventElapsedTime(&ms, e.second.first, e.second.second));
      tot[e.first] += ms;
      cnt[e.first] += 1;
      cudaEventDestroy(e.second.first);
      cudaEventDestroy(e.second.second);
    }
    for (int c = 0; c < K_NCLASS && written < cap; ++c) {
      if (!cnt[c]) continue;
      names[written] = kNames[c];
      ms_per_step[written] = tot[c] / nsteps;
      if (launches_per_step) launches_per_step[written] = cnt[c] / nsteps;
      ++written;
    }
    return TTSH_OK;
  });
  return rc ? -rc : written;
}

int ttsh_num_groups(const ttsh_sim* s) {
  if (!s) return 0;
  return s->precision == 32 ? (int)s->ef.groups.size() : (int)s->ed.groups.size();
}

int ttsh_get_tuning(const ttsh_sim* s, int group, ttsh_tuning* out) {
  if (!s || !out) return set_error(TTSH_E_INVALID, "null argument");
  if (group < 0 || group >= ttsh_num_groups(s)) return set_error(TTSH_E_INVALID, "group out of range");
  if (s->precision == 32) get_tuning(s, s->ef, group, out);
  else get_tuning(s, s->ed, group, out);
  return TTSH_OK;
}

int ttsh_set_tuning(ttsh_sim* s, int group, const ttsh_tuning* in) {
  if (!s || !in) return set_error(TTSH_E_INVALID, "null argument");
  if (group < 0 || group >= ttsh_num_groups(s)) return set_error(TTSH_E_INVALID, "group out of range");
  return guarded([&]() -> int {
    CK(cudaSetDevice(s->device));
    std::string err;
    s->with_engine([&](auto& E) { err = check_tuning(s, E.groups[group], *in); });
    if (!err.empty()) return set_error(TTSH_E_INVALID, err);
    CK(cudaStreamSynchronize(s->stream));
    s->with_engine([&](auto& E) { apply_tuning(s, E, group, *in); });
    capture_graphs(s);
    return TTSH_OK;
  });
}

int ttsh_autotune(ttsh_sim* s, const char* cache_path) {
  if (!s) return set_error(TTSH_E_INVALID, "null argument");
  return guarded([&]() -> int {
    CK(cudaSetDevice(s->device));
    CK(cudaStreamSynchronize(s->stream));
    std::map<std::string, ttsh_tuning> cache;
    if (cache_path) cache = read_cache(cache_path);
    int rc = TTSH_OK;
    s->with_engine([&](auto& E) {
      for (size_t g = 0; g < E.groups.size() && rc == TTSH_OK; ++g) {
        const std::string key = tune_key(s, E.groups[g].N, E.groups[g].n);
        auto it = cache.find(key);
        if (it != cache.end()) {
          ttsh_tuning t = it->second;
          t.N = E.groups[g].N;
          t.n = E.groups[g].n;
          const std::string err = check_tuning(s, E.groups[g], t);
          if (err.empty()) {
            apply_tuning(s, E, g, t);
            continue;
          }
        }
        ttsh_tuning t{};
        tune_group(s, E, g, &t);
        if (cache_path) append_cache(cache_path, key, t);
      }
    });
    capture_graphs(s);
    return rc;
  });
}

const char* ttsh_strerror(int code) {
  switch (code) {
    case TTSH_OK: return "ok";
    case TTSH_E_INVALID: return "invalid argument";
    case TTSH_E_IO: return "i/o error";
    case TTSH_E_PARSE: return "Error while reading the input file!";
    case TTSH_E_CUDA: return "CUDA error";
    case TTSH_E_NODEVICE: return "no CUDA device";
    case TTSH_E_NOMEM: return "out of memory";
    case TTSH_E_UNSTABLE: return "non-finite state";
    case TTSH_E_UNSUPPORTED: return "unsupported size or option";
    default: return "unknown error";
  }
}

const char* ttsh_last_error(void) { return g_last_error.c_str(); }

}  // extern "C"
