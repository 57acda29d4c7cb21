// ttsh_oracle.cpp — FP64 CPU restatement of the TTSH3D explicit step.
//
// TEST INFRASTRUCTURE ONLY. This file is the checker that the CUDA path in
// libttsh is compared against; it is never linked into the product and the
// product never calls it. Only tests/, __graft_entry__.smoke() and bench.py's
// cpu_baseline / reference legs may load it.
//
// What it restates (file:line relative to bacterial_droplet_12-16/ of the
// reference project, TTSH3D.cu):
//   * EEuler()                :347-359  step order (RHS, u*/P*, two projections, correction)
//   * getTempVari_1           :537-558  D_a P_b and |grad phi|^2
//   * getTempVari_2           :561-605  mu_0, P2, mu_b, sigma_ab, A_ab (with the integer-division
//                                       zeros 1/2, 1/28, 1/3 -> the D.P, Omega.P, L(dP) and trace
//                                       terms vanish; quirk Q1)
//   * getDtF                  :608-632  d/dt of u, P, phi
//   * getVStar / getVNew      :471-516  provisional fields and pressure-gradient correction
//   * getP / getStream        :635-691  divergence / dt0, forward FFT, -F/k2, inverse FFT, Re/N^3
//   * initPoissonSolver       :1088-1124 continuous k^2 with k2[0] = 1 (quirk Q5)
//   * d1{x,y,z}CO2I3D, laplaceCO2I3D :3280-3343 stencils, same neighbour order and constants
//   * BounPeriU               :1422-1607 periodic halo; restated as index wrap, except for the
//                                       divergence of u*/P*, whose wrapped neighbours come from
//                                       the previous step's u*/P* (quirk Q2: the halo is
//                                       refreshed at the start of getRHS, :369-371, :405-407,
//                                       before getVStar rewrites the interior)
// Build-defined extension (absent from the reference): the active stress
// -zeta * D_a(phi P_a P_b) added to d/dt u_b; it is skipped when zeta == 0 so
// that the zeta = 0 step is the reference step.
//
// Arithmetic is FP64 everywhere. Compile with -ffp-contract=off so that x86
// and aarch64 builds give identical bits (no reductions depend on thread count).
#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdint>
#include <cstring>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef std::complex<double> cplx;

extern "C" {

typedef struct {
  int N;
  double h, dt;
  double mu, cA, alpha, beta, eta, La, kappa, lambda0, aPhi, kPhi, gamma, A;
  double zeta;
  int k2_mode;     // 0: continuous k^2 with k2[0]=1 (reference), 1: modified wavenumber of D_a
  int stale_halo;  // 1: quirk Q2 (wrapped neighbours of u*/P* in the divergence from previous step)
} orc_params;

typedef struct {
  double *phi, *px, *py, *pz, *vx, *vy, *vz;
  double *vxs, *vys, *vzs, *pxs, *pys, *pzs;  // u*, P* (previous-step values on entry)
  double *pv, *pp;                             // pressures (outputs)
} orc_state;

}  // extern "C"

namespace {

const double kPi = 3.1415926535897932384626433832795;

inline int wrap(int a, int N) { return a < 0 ? a + N : (a >= N ? a - N : a); }

// Neighbour accessor: value of f at (x+dx, y+dy, z+dz) with periodic wrap.
// If `old` is non-null, wrapped reads come from `old` instead (quirk Q2).
struct Nb {
  const double* f;
  const double* old;
  int N, x, y, z;
  inline double operator()(int dx, int dy, int dz) const {
    int X = x + dx, Y = y + dy, Z = z + dz;
    bool wrapped = (X < 0 || X >= N || Y < 0 || Y >= N || Z < 0 || Z >= N);
    X = wrap(X, N); Y = wrap(Y, N); Z = wrap(Z, N);
    size_t i = ((size_t)Z * N + Y) * N + X;
    return (wrapped && old) ? old[i] : f[i];
  }
};

// Accessor for the pointwise product phi * P_a * P_b (the build-defined active stress).
struct ProdNb {
  const double *phi, *pa, *pb;
  int N, x, y, z;
  inline double operator()(int dx, int dy, int dz) const {
    int X = wrap(x + dx, N), Y = wrap(y + dy, N), Z = wrap(z + dz, N);
    size_t j = ((size_t)Z * N + Y) * N + X;
    return phi[j] * pa[j] * pb[j];
  }
};

// d1xCO2I3D (TTSH3D.cu:3280-3295): same neighbour order and constants.
template <class Acc>
inline double d1x(const Acc& F, double h) {
  return 1.0 / (2.0 * h) *
         (16.0 / 36 * (F(1, 0, 0) - F(-1, 0, 0)) +
          4.0 / 36 * (F(1, 0, 1) + F(1, 0, -1) + F(1, 1, 0) + F(1, -1, 0) - F(-1, 0, 1) - F(-1, 0, -1) -
                      F(-1, 1, 0) - F(-1, -1, 0)) +
          1.0 / 36 * (F(1, 1, 1) + F(1, -1, 1) + F(1, 1, -1) + F(1, -1, -1) - F(-1, 1, 1) - F(-1, -1, 1) -
                      F(-1, 1, -1) - F(-1, -1, -1)));
}
// d1yCO2I3D (TTSH3D.cu:3298-3312)
template <class Acc>
inline double d1y(const Acc& F, double h) {
  return 1.0 / (2.0 * h) *
         (16.0 / 36 * (F(0, 1, 0) - F(0, -1, 0)) +
          4.0 / 36 * (F(0, 1, 1) + F(0, 1, -1) + F(1, 1, 0) + F(-1, 1, 0) - F(0, -1, 1) - F(0, -1, -1) -
                      F(1, -1, 0) - F(-1, -1, 0)) +
          1.0 / 36 * (F(1, 1, 1) + F(-1, 1, 1) + F(1, 1, -1) + F(-1, 1, -1) - F(1, -1, 1) - F(-1, -1, 1) -
                      F(1, -1, -1) - F(-1, -1, -1)));
}
// d1zCO2I3D (TTSH3D.cu:3315-3328)
template <class Acc>
inline double d1z(const Acc& F, double h) {
  return 1.0 / (2.0 * h) *
         (16.0 / 36 * (F(0, 0, 1) - F(0, 0, -1)) +
          4.0 / 36 * (F(1, 0, 1) + F(-1, 0, 1) + F(0, 1, 1) + F(0, -1, 1) - F(1, 0, -1) - F(-1, 0, -1) -
                      F(0, 1, -1) - F(0, -1, -1)) +
          1.0 / 36 * (F(1, 1, 1) + F(1, -1, 1) + F(-1, 1, 1) + F(-1, -1, 1) - F(1, 1, -1) - F(1, -1, -1) -
                      F(-1, 1, -1) - F(-1, -1, -1)));
}
// laplaceCO2I3D (TTSH3D.cu:3331-3343)
template <class Acc>
inline double lap(const Acc& F, double h) {
  return 1.0 / (12 * h * h) *
             (F(1, 1, -1) + F(1, -1, -1) + F(-1, 1, -1) + F(-1, -1, -1) + F(1, 1, 1) + F(1, -1, 1) +
              F(-1, 1, 1) + F(-1, -1, 1)) +
         2.0 / (3 * h * h) * (F(0, 0, -1) + F(0, 0, 1) + F(-1, 0, 0) + F(1, 0, 0) + F(0, -1, 0) + F(0, 1, 0)) -
         14.0 / (3 * h * h) * F(0, 0, 0);
}

template <class Acc>
inline double dA(int a, const Acc& F, double h) { return a == 0 ? d1x(F, h) : (a == 1 ? d1y(F, h) : d1z(F, h)); }

// ---------------------------------------------------------------------------
// Mixed-radix Stockham FFT (radix 4, 2, 3, 5, and a plain DFT for any other
// prime factor). Sign -1 = forward (cuFFT CUFFT_FORWARD), +1 = inverse,
// both unnormalised, as cufftExecZ2Z.
struct Plan1D {
  int N;
  std::vector<int> radix;
  std::vector<cplx> w;  // w[k] = exp(-2 pi i k / N)
  explicit Plan1D(int n) : N(n) {
    int m = n;
    while (m % 4 == 0) { radix.push_back(4); m /= 4; }
    while (m % 2 == 0) { radix.push_back(2); m /= 2; }
    for (int p = 3; m > 1; p += 2)
      while (m % p == 0) { radix.push_back(p); m /= p; }
    w.resize(n);
    for (int k = 0; k < n; ++k) {
      double a = -2.0 * kPi * (double)k / (double)n;
      w[k] = cplx(std::cos(a), std::sin(a));
    }
  }
  inline cplx tw(long k, int sign) const {
    cplx t = w[(size_t)(k % N)];
    return sign < 0 ? t : std::conj(t);
  }
  // In-place transform of `a` (length N) using scratch `b` (length N).
  void run(cplx* a, cplx* b, int sign) const {
    cplx* src = a;
    cplx* dst = b;
    int Ns = 1;
    cplx v[64];
    for (int R : radix) {
      int M = N / R;
      for (int j = 0; j < M; ++j) {
        int k = j % Ns;
        long tstep = (long)k * (N / (Ns * R));
        for (int r = 0; r < R; ++r) v[r] = src[j + r * M] * tw((long)r * tstep, sign);
        cplx o[64];
        for (int q = 0; q < R; ++q) {
          cplx s = 0;
          for (int r = 0; r < R; ++r) s += v[r] * tw((long)((q * r) % R) * (N / R), sign);
          o[q] = s;
        }
        int d = (j / Ns) * Ns * R + k;
        for (int r = 0; r < R; ++r) dst[d + r * Ns] = o[r];
      }
      std::swap(src, dst);
      Ns *= R;
    }
    if (src != a) std::memcpy(a, src, sizeof(cplx) * N);
  }
};

// 3D FFT over an N^3 array with x fastest: a DFT along each axis.
void fft3(cplx* data, int N, int sign) {
  Plan1D plan(N);
  size_t N2 = (size_t)N * N;
  for (int axis = 0; axis < 3; ++axis) {
    size_t stride = axis == 0 ? 1 : (axis == 1 ? (size_t)N : N2);
#pragma omp parallel
    {
      std::vector<cplx> line(N), scr(N);
#pragma omp for schedule(static)
      for (long l = 0; l < (long)N2; ++l) {
        size_t base;
        if (axis == 0) base = (size_t)l * N;                         // (z,y) rows
        else if (axis == 1) base = (size_t)(l / N) * N2 + (l % N);   // (z,x)
        else base = (size_t)l;                                       // (y,x)
        for (int e = 0; e < N; ++e) line[e] = data[base + e * stride];
        plan.run(line.data(), scr.data(), sign);
        for (int e = 0; e < N; ++e) data[base + e * stride] = line[e];
      }
    }
  }
}

// Poisson multiplier at frequency (mx,my,mz), following initPoissonSolver
// (TTSH3D.cu:1088-1124) in mode 0; mode 1 uses the symbol of the discrete
// gradient D_a, i sin(k_a h)/h * prod_{b!=a} (2 + cos k_b h)/3, so that the
// projection is exactly solenoidal for D (modes where that symbol vanishes
// are set to zero).
inline double kwave(int m, int N, double h) {
  double k = 2 * kPi * m / (N * h + 0.0);
  if (m >= N / 2) k = 2 * kPi * (m - N) / (N * h + 0.0);
  return k;
}

void poisson_divide(cplx* F, int N, double h, int mode) {
  std::vector<double> kk(N), S(N), C(N);
  for (int m = 0; m < N; ++m) {
    kk[m] = kwave(m, N, h);
    S[m] = std::sin(kk[m] * h) / h;
    C[m] = (2.0 + std::cos(kk[m] * h)) / 3.0;
  }
#pragma omp parallel for schedule(static)
  for (long zy = 0; zy < (long)N * N; ++zy) {
    int z = (int)(zy / N), y = (int)(zy % N);
    for (int x = 0; x < N; ++x) {
      size_t i = (size_t)zy * N + x;
      if (mode == 0) {
        double k2 = kk[x] * kk[x] + kk[y] * kk[y] + kk[z] * kk[z];
        if (i == 0) k2 = 1;  // TTSH3D.cu:1120
        F[i] = cplx(-F[i].real() / k2, -F[i].imag() / k2);
      } else {
        double Kx = S[x] * C[y] * C[z], Ky = C[x] * S[y] * C[z], Kz = C[x] * C[y] * S[z];
        double K2 = Kx * Kx + Ky * Ky + Kz * Kz;
        if (K2 < 1e-24) F[i] = 0;
        else F[i] = cplx(-F[i].real() / K2, -F[i].imag() / K2);
      }
    }
  }
}

struct Work {
  int N;
  size_t n;
  std::vector<double> dP[9], mu0, mu[3], sig[9], dtv[3], dtp[3], dtphi, old[6];
  std::vector<cplx> F;
  explicit Work(int N_) : N(N_), n((size_t)N_ * N_ * N_) {
    for (auto& a : dP) a.resize(n);
    mu0.resize(n);
    for (auto& a : mu) a.resize(n);
    for (auto& a : sig) a.resize(n);
    for (auto& a : dtv) a.resize(n);
    for (auto& a : dtp) a.resize(n);
    dtphi.resize(n);
    for (auto& a : old) a.resize(n);
    F.resize(n);
  }
};

#define SITE_LOOP(N)                                   \
  _Pragma("omp parallel for schedule(static)")         \
  for (long zy = 0; zy < (long)(N) * (N); ++zy)        \
    for (int x = 0, z = (int)(zy / (N)), y = (int)(zy % (N)); x < (N); ++x)

// getP (TTSH3D.cu:635-651) for one vector field X* -> pressure p.
void project(const orc_params& p, Work& w, const double* const Xs[3], const double* const Xold[3], double* out) {
  const int N = p.N;
  const double h = p.h;
  SITE_LOOP(N) {
    size_t i = ((size_t)z * N + y) * N + x;
    const double* o0 = p.stale_halo ? Xold[0] : nullptr;
    const double* o1 = p.stale_halo ? Xold[1] : nullptr;
    const double* o2 = p.stale_halo ? Xold[2] : nullptr;
    Nb A{Xs[0], o0, N, x, y, z}, B{Xs[1], o1, N, x, y, z}, C{Xs[2], o2, N, x, y, z};
    // getStream mode 0 (TTSH3D.cu:664-670)
    w.F[i] = cplx((d1x(A, h) + d1y(B, h) + d1z(C, h)) / p.dt, 0.0);
  }
  fft3(w.F.data(), N, -1);
  poisson_divide(w.F.data(), N, h, p.k2_mode);
  fft3(w.F.data(), N, +1);
  const double NNN = (double)(N * N * N);
  for (size_t i = 0; i < w.n; ++i) out[i] = w.F[i].real() / NNN;  // getStream mode 2
}

void one_step(const orc_params& p, orc_state& s, Work& w) {
  const int N = p.N;
  const double h = p.h, dt = p.dt;
  const double* P[3] = {s.px, s.py, s.pz};
  const double* V[3] = {s.vx, s.vy, s.vz};

  // getTempVari_1 (TTSH3D.cu:537-558): dP[a*3+b] = D_a P_b.
  SITE_LOOP(N) {
    size_t i = ((size_t)z * N + y) * N + x;
    for (int b = 0; b < 3; ++b) {
      Nb F{P[b], nullptr, N, x, y, z};
      for (int a = 0; a < 3; ++a) w.dP[a * 3 + b][i] = dA(a, F, h);
    }
  }
  // getTempVari_2 (TTSH3D.cu:561-605). D.P, Omega.P (1/2 -> 0), the 1/28 Laplacian and the
  // 1/3 trace term are integer-division zeros in the reference and are omitted.
  SITE_LOOP(N) {
    size_t i = ((size_t)z * N + y) * N + x;
    Nb Fphi{s.phi, nullptr, N, x, y, z};
    double ph = s.phi[i];
    w.mu0[i] = p.aPhi * 2 * (ph - 3 * ph * ph + 2 * ph * ph * ph) - p.kPhi * lap(Fphi, h);
    for (int b = 0; b < 3; ++b) {
      Nb F{P[b], nullptr, N, x, y, z};
      w.mu[b][i] = ph * P[b][i] + p.La * p.La * lap(F, h);
    }
    for (int k = 0; k < 9; ++k) w.sig[k][i] = ph * w.dP[k][i];
  }
  // getDtF (TTSH3D.cu:608-632)
  SITE_LOOP(N) {
    size_t i = ((size_t)z * N + y) * N + x;
    Nb Fphi{s.phi, nullptr, N, x, y, z};
    double dphi[3] = {d1x(Fphi, h), d1y(Fphi, h), d1z(Fphi, h)};
    double vx = s.vx[i], vy = s.vy[i], vz = s.vz[i];
    double px = s.px[i], py = s.py[i], pz = s.pz[i], ph = s.phi[i];
    double P2 = px * px + py * py + pz * pz;
    double dPhi2 = dphi[0] * dphi[0] + dphi[1] * dphi[1] + dphi[2] * dphi[2];
    double Am[3][3];
    for (int a = 0; a < 3; ++a)
      for (int b = 0; b < 3; ++b) Am[a][b] = dphi[a] * dphi[b];
    for (int b = 0; b < 3; ++b) {
      Nb Fv{V[b], nullptr, N, x, y, z};
      Nb S0{w.sig[0 * 3 + b].data(), nullptr, N, x, y, z};
      Nb S1{w.sig[1 * 3 + b].data(), nullptr, N, x, y, z};
      Nb S2{w.sig[2 * 3 + b].data(), nullptr, N, x, y, z};
      double r = -vx * d1x(Fv, h) - vy * d1y(Fv, h) - vz * d1z(Fv, h) + p.mu * lap(Fv, h) +
                 w.mu0[i] * dphi[b] + p.cA * (d1x(S0, h) + d1y(S1, h) + d1z(S2, h));
      if (p.zeta != 0.0) {
        // -zeta * sum_a D_a (phi P_a P_b), the stencil applied to the product field.
        ProdNb Q0{s.phi, P[0], P[b], N, x, y, z}, Q1{s.phi, P[1], P[b], N, x, y, z}, Q2{s.phi, P[2], P[b], N, x, y, z};
        r = r - p.zeta * (d1x(Q0, h) + d1y(Q1, h) + d1z(Q2, h));
      }
      w.dtv[b][i] = r;
    }
    double pb[3] = {px, py, pz};
    for (int b = 0; b < 3; ++b) {
      Nb Fp{P[b], nullptr, N, x, y, z};
      Nb Fmu{w.mu[b].data(), nullptr, N, x, y, z};
      double dxp = d1x(Fp, h), dyp = d1y(Fp, h), dzp = d1z(Fp, h);
      double cub;  // the reference's P_b * |P|^2 written out term by term
      if (b == 0) cub = px * px * px + px * py * py + px * pz * pz;
      else if (b == 1) cub = px * py * px + py * py * py + py * pz * pz;
      else cub = px * pz * px + py * pz * py + pz * pz * pz;
      double Ab = Am[0][b] * px + Am[1][b] * py + Am[2][b] * pz;
      // OP_b + kappa*phi*DP_b are exact zeros (Q1) and are omitted.
      w.dtp[b][i] = -vx * dxp - vy * dyp - vz * dzp - p.alpha * ph * pb[b] - p.beta * P2 * pb[b] +
                    p.eta * lap(Fmu, h) - p.lambda0 * (px * dxp + py * dyp + pz * dzp) -
                    p.A * (dPhi2 * cub + std::sqrt(P2) * Ab);
    }
    Nb Fmu0{w.mu0.data(), nullptr, N, x, y, z};
    w.dtphi[i] = -vx * dphi[0] - vy * dphi[1] - vz * dphi[2] + p.gamma * (lap(Fmu0, h));
  }
  // Previous-step u*/P* (the halo contents seen by getStream mode 0 in the reference).
  double* Xs[6] = {s.vxs, s.vys, s.vzs, s.pxs, s.pys, s.pzs};
  if (p.stale_halo)
    for (int c = 0; c < 6; ++c) std::memcpy(w.old[c].data(), Xs[c], sizeof(double) * w.n);
  // getVStar (TTSH3D.cu:471-491)
  SITE_LOOP(N) {
    size_t i = ((size_t)z * N + y) * N + x;
    for (int b = 0; b < 3; ++b) {
      Xs[b][i] = V[b][i] + dt * w.dtv[b][i];
      Xs[3 + b][i] = P[b][i] + dt * w.dtp[b][i];
    }
  }
  // getP(f,0), getP(f,1) (TTSH3D.cu:353-354)
  {
    const double* us[3] = {s.vxs, s.vys, s.vzs};
    const double* uo[3] = {w.old[0].data(), w.old[1].data(), w.old[2].data()};
    project(p, w, us, uo, s.pv);
    const double* ps[3] = {s.pxs, s.pys, s.pzs};
    const double* po[3] = {w.old[3].data(), w.old[4].data(), w.old[5].data()};
    project(p, w, ps, po, s.pp);
  }
  // getVNew (TTSH3D.cu:494-516)
  SITE_LOOP(N) {
    size_t i = ((size_t)z * N + y) * N + x;
    Nb Fv{s.pv, nullptr, N, x, y, z}, Fp{s.pp, nullptr, N, x, y, z};
    s.vx[i] = s.vxs[i] - dt * d1x(Fv, h);
    s.vy[i] = s.vys[i] - dt * d1y(Fv, h);
    s.vz[i] = s.vzs[i] - dt * d1z(Fv, h);
    s.px[i] = s.pxs[i] - dt * d1x(Fp, h);
    s.py[i] = s.pys[i] - dt * d1y(Fp, h);
    s.pz[i] = s.pzs[i] - dt * d1z(Fp, h);
    s.phi[i] = s.phi[i] + dt * w.dtphi[i];
  }
}

}  // namespace

extern "C" {

int orc_set_threads(int n) {
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
  return omp_get_max_threads();
#else
  (void)n;
  return 1;
#endif
}

int orc_step(const orc_params* p, orc_state* s, int nsteps) {
  if (!p || !s || p->N < 4 || nsteps < 0) return 1;
  Work w(p->N);
  for (int t = 0; t < nsteps; ++t) one_step(*p, *s, w);
  return 0;
}

// Single stencil applications (for symbol tests). axis 0,1,2 = D_x, D_y, D_z; 3 = L.
void orc_stencil(const double* f, int N, double h, int op, double* out) {
  SITE_LOOP(N) {
    size_t i = ((size_t)z * N + y) * N + x;
    Nb F{f, nullptr, N, x, y, z};
    out[i] = op < 3 ? dA(op, F, h) : lap(F, h);
  }
}

// In-place 3D FFT of N^3 interleaved complex doubles. sign -1 forward, +1 inverse (unnormalised).
void orc_fft3(double* data, int N, int sign) { fft3(reinterpret_cast<cplx*>(data), N, sign); }

// One projection: pressure p from X* (no stale halo), as getP.
void orc_project(const double* xs, const double* ys, const double* zs, int N, double h, double dt, int k2_mode,
                 double* out) {
  orc_params p{};
  p.N = N; p.h = h; p.dt = dt; p.k2_mode = k2_mode; p.stale_halo = 0;
  Work w(N);
  const double* X[3] = {xs, ys, zs};
  const double* O[3] = {nullptr, nullptr, nullptr};
  project(p, w, X, O, out);
}

// The droplet initial condition of the benchmark workloads (a build-defined extension of the
// reference, whose InitConf has no seed, radius or width; TTSH3D.cu:801-824): phi =
// (1 - tanh((r - R)/xi))/2 about the box centre; inside (phi > 0.5) a unit direction uniform on
// the sphere from a counter-based generator (splitmix64 of seed and site), optionally tilted by
// Gaussian angular noise; three Jacobi passes (mean of the site and its 6 face neighbours,
// periodic); P zeroed again where phi <= 0.5. The same draws and operation order as libttsh's
// ttsh_init_droplet, so both give the same bits with the same compiler flags; the timed
// reference arm builds its input with this one and never loads libttsh.
static inline uint64_t orc_splitmix64(uint64_t x) {
  x += 0x9E3779B97F4A7C15ull;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  return x ^ (x >> 31);
}
static inline double orc_uni(uint64_t seed, uint64_t idx, uint64_t k) {
  return (double)(orc_splitmix64(orc_splitmix64(seed) ^ (idx * 8 + k)) >> 11) * (1.0 / 9007199254740992.0);
}

int orc_init_droplet(int N, double h, double R, double xi, uint64_t seed, double angular_noise, double* phi,
                     double* P) {
  if (N < 4 || !(h > 0) || !(xi > 0) || !phi || !P) return 1;
  const size_t n = (size_t)N * N * N;
  const double c = N / 2.0, twopi = 6.283185307179586476925286766559;
  std::vector<double> Q(3 * n, 0.0), T(3 * n);
  for (int z = 0; z < N; ++z)
    for (int y = 0; y < N; ++y)
      for (int x = 0; x < N; ++x) {
        const size_t i = ((size_t)z * N + y) * N + x;
        const double dx = x - c, dy = y - c, dz = z - c;
        phi[i] = 0.5 * (1.0 - std::tanh((h * std::sqrt(dx * dx + dy * dy + dz * dz) - R) / xi));
        if (!(phi[i] > 0.5)) continue;
        const double cz = 1.0 - 2.0 * orc_uni(seed, i, 0), az = twopi * orc_uni(seed, i, 1);
        const double s = std::sqrt(std::max(0.0, 1.0 - cz * cz));
        double v[3] = {s * std::cos(az), s * std::sin(az), cz};
        if (angular_noise > 0) {
          double g[3], w[3], nn = 0;
          for (int k = 0; k < 3; ++k) {
            const double u1 = 1.0 - orc_uni(seed, i, 2 + k), u2 = orc_uni(seed, i, 5 + (k % 3));
            g[k] = std::sqrt(-2.0 * std::log(u1)) * std::cos(twopi * u2);
          }
          const double gp = g[0] * v[0] + g[1] * v[1] + g[2] * v[2];
          for (int k = 0; k < 3; ++k) {
            w[k] = v[k] + angular_noise * (g[k] - gp * v[k]);
            nn += w[k] * w[k];
          }
          nn = std::sqrt(nn);
          for (int k = 0; k < 3; ++k) v[k] = w[k] / nn;
        }
        for (int k = 0; k < 3; ++k) Q[k * n + i] = v[k];
      }
  for (int pass = 0; pass < 3; ++pass) {
    for (int k = 0; k < 3; ++k) {
      const double* a = &Q[k * n];
      double* b = &T[k * n];
      for (int z = 0; z < N; ++z)
        for (int y = 0; y < N; ++y)
          for (int x = 0; x < N; ++x) {
            auto at = [&](int X, int Y, int Z) { return a[((size_t)wrap(Z, N) * N + wrap(Y, N)) * N + wrap(X, N)]; };
            b[((size_t)z * N + y) * N + x] = (at(x, y, z) + at(x - 1, y, z) + at(x + 1, y, z) + at(x, y - 1, z) +
                                              at(x, y + 1, z) + at(x, y, z - 1) + at(x, y, z + 1)) / 7.0;
          }
    }
    Q.swap(T);
  }
  for (size_t i = 0; i < n; ++i)
    for (int k = 0; k < 3; ++k) P[k * n + i] = phi[i] > 0.5 ? Q[k * n + i] : 0.0;
  return 0;
}

// FP64 mass sum(phi) h^3, serial (order fixed).
double orc_mass(const double* phi, int N, double h) {
  double s = 0;
  size_t n = (size_t)N * N * N;
  for (size_t i = 0; i < n; ++i) s += phi[i];
  return s * h * h * h;
}

// max |sum_a D_a u_a| over the grid.
double orc_max_div(const double* vx, const double* vy, const double* vz, int N, double h) {
  double m = 0;
  for (int z = 0; z < N; ++z)
    for (int y = 0; y < N; ++y)
      for (int x = 0; x < N; ++x) {
        Nb A{vx, nullptr, N, x, y, z}, B{vy, nullptr, N, x, y, z}, C{vz, nullptr, N, x, y, z};
        double d = std::fabs(d1x(A, h) + d1y(B, h) + d1z(C, h));
        if (d > m) m = d;
      }
  return m;
}

}  // extern "C"
