// io.cpp — host-side boundary of libttsh: the input.dat reader, the snapshot
// writer and the build-defined initial condition. No CUDA here.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <memory>
#include <random>
#include <string>
#include <thread>
#include <vector>

#include "../../include/ttsh.h"
#include "internal.h"

using ttsh::set_error;

namespace {

// printf "%.15f" of x, written at p (at least F15_MAX bytes of room); returns the end. printf
// prints the exact binary value of x rounded to 15 decimals, ties to even. For |x| < 2^13 that
// value is computed exactly: x = m 2^e with m < 2^53 and e <= -40, so m 10^15 < 2^103 fits
// 128-bit integers and the rounding of m 10^15 / 2^-e is decided on the exact remainder. The sign
// is printed whenever x's sign bit is set, as printf does for -0.0 and for negative values that
// round to zero. Larger magnitudes, infinities and NaNs go to snprintf itself.
constexpr int F15_MAX = 340;  // "-" + 309 integer digits + "." + 15 decimals + NUL, rounded up
char* put_f15(char* p, double x) {
  uint64_t bits;
  std::memcpy(&bits, &x, sizeof bits);
  const int be = (int)((bits >> 52) & 0x7ff);
  if (be >= 1023 + 13) return p + std::snprintf(p, F15_MAX, "%.15f", x);  // |x| >= 2^13, inf, nan
  constexpr uint64_t P15 = 1000000000000000ull;
  uint64_t m = bits & ((1ull << 52) - 1);
  int e;
  if (be == 0) {
    e = -1074;  // subnormal
  } else {
    m |= 1ull << 52;
    e = be - 1075;  // <= -40 here
  }
  uint64_t r;  // |x| 10^15 rounded to an integer, ties to even (< 2^13 10^15 < 2^63)
  if (-e >= 128) {
    r = 0;  // |x| 10^15 < 2^103 / 2^128
  } else {
    const unsigned __int128 v = (unsigned __int128)m * P15;
    const int s = -e;
    const unsigned __int128 q = v >> s;
    const unsigned __int128 rem = v - (q << s);
    const unsigned __int128 half = (unsigned __int128)1 << (s - 1);
    r = (uint64_t)q + ((rem > half || (rem == half && (q & 1))) ? 1 : 0);
  }
  if (bits >> 63) *p++ = '-';
  const uint64_t ip = r / P15;
  uint64_t fp = r - ip * P15;
  // integer part (< 2^13 + 1)
  char ib[8];
  int ni = 0;
  uint64_t t = ip;
  do {
    ib[ni++] = (char)('0' + t % 10);
    t /= 10;
  } while (t);
  while (ni) *p++ = ib[--ni];
  *p++ = '.';
  for (int k = 14; k >= 0; --k) {
    p[k] = (char)('0' + fp % 10);
    fp /= 10;
  }
  return p + 15;
}

}  // namespace

extern "C" {

// GetInput (TTSH3D.cu:696-752): the same 33 extractions, in the same order and into
// the same types, so a file the reference accepts is accepted here and vice versa.
int ttsh_read_input(const char* path, ttsh_input* o) {
  if (!path || !o) return set_error(TTSH_E_INVALID, "ttsh_read_input: null argument");
  std::ifstream f(path);
  if (!f.is_open()) return set_error(TTSH_E_IO, std::string("cannot open ") + path);
  std::memset(o, 0, sizeof(*o));
  o->ReadSuccess = 0;
  f >> o->TimeScheme >> o->RKStage >> o->ExplImpi >> o->AdapTime >> o->ExpoData >> o->InitCond >> o->isSimplified >>
      o->checkUnStable;
  f >> o->Nx >> o->Ny >> o->Nz >> o->Nb;
  f >> o->h >> o->dt0 >> o->T0 >> o->Ts >> o->dte >> o->dtVarC >> o->dtMax;
  f >> o->mu >> o->cA >> o->alpha >> o->beta >> o->eta >> o->La >> o->kappa >> o->lambda0 >> o->aPhi >> o->kPhi >>
      o->gamma >> o->A >> o->init0;
  f >> o->ReadSuccess;
  if (o->ReadSuccess != TTSH_READ_SUCCESS)
    return set_error(TTSH_E_PARSE, "Error while reading the input file!");  // TTSH3D.cu:750
  return TTSH_OK;
}

// run_cuda.pl:7-44 (the parameters it writes to input.dat).
void ttsh_default_input(ttsh_input* o) {
  if (!o) return;
  std::memset(o, 0, sizeof(*o));
  o->TimeScheme = 1; o->RKStage = 16; o->ExplImpi = 1; o->AdapTime = 0; o->ExpoData = 1; o->InitCond = 1;
  o->isSimplified = 1; o->checkUnStable = 0;
  o->Nx = o->Ny = o->Nz = 64; o->Nb = 3;
  o->h = 1; o->dt0 = 0.002; o->T0 = 0; o->Ts = 1000; o->dte = 10; o->dtVarC = 0.01; o->dtMax = 0.000005;
  o->mu = 1; o->cA = -1; o->alpha = -0.02; o->beta = 4.366; o->eta = -0.187; o->La = 1; o->kappa = -0.364;
  o->lambda0 = 9; o->aPhi = 1; o->kPhi = 1; o->gamma = 1; o->A = 0; o->init0 = 0.0001;
  o->ReadSuccess = TTSH_READ_SUCCESS;
}

int ttsh_struct_size(int which) {
  switch (which) {
    case 0: return (int)sizeof(ttsh_input);
    case 1: return (int)sizeof(ttsh_ext);
    case 2: return (int)sizeof(ttsh_stats);
    case 3: return (int)sizeof(ttsh_tuning);
    default: return -1;
  }
}

void ttsh_default_ext(ttsh_ext* e) {
  if (!e) return;
  std::memset(e, 0, sizeof(*e));
  e->zeta = 0; e->R = 16; e->xi = 2; e->seed = 0; e->precision = 64;
  e->k2_mode = TTSH_K2_REFERENCE; e->quirks = TTSH_QUIRK_STALE_HALO;
}

// ExpoConf's text layout (TTSH3D.cu:966-1013): y outer, x, z inner; ExpoData == 1 writes
// "vx vy vz px py pz phi\n" and ExpoData == -1 writes "vx vy " (no newline), each value as
// `fixed << setprecision(15)`, i.e. printf "%.15f". Lines are formatted in parallel and
// written in order.
int ttsh_format_conf(int N, int expo_data, const double* phi, const double* P, const double* u, const char* path) {
  if (N <= 0 || !path) return set_error(TTSH_E_INVALID, "ttsh_format_conf: bad arguments");
  if (expo_data == 1 && (!phi || !P || !u)) return set_error(TTSH_E_INVALID, "ttsh_format_conf: null field");
  if (expo_data == -1 && !u) return set_error(TTSH_E_INVALID, "ttsh_format_conf: null field");
  FILE* fp = std::fopen(path, "wb");
  if (!fp) return set_error(TTSH_E_IO, std::string("cannot open ") + path);
  if (expo_data != 1 && expo_data != -1) {  // the reference's loop writes nothing
    std::fclose(fp);
    return TTSH_OK;
  }
  const size_t n = (size_t)N * N * N;
  const size_t NN = (size_t)N * N;
  unsigned nth = std::max(1u, std::min(64u, std::thread::hardware_concurrency()));
  // Each round formats nth chunks of consecutive y-planes (the outer loop); a chunk holds about 8 MB
  // of text at most, so memory stays bounded (two rounds). A writer thread writes round k in order
  // while round k + 1 is formatted.
  const int chunk_rows = std::max(1, (int)std::min<size_t>((size_t)N / nth, (size_t)(8u << 20) / (NN * 140)));
  int err = 0;
  std::vector<std::string> bufs[2] = {std::vector<std::string>(nth), std::vector<std::string>(nth)};
  std::thread writer;
  int round = 0;
  for (int y0 = 0; y0 < N; y0 += chunk_rows * (int)nth, ++round) {
    std::vector<std::string>& cur = bufs[round & 1];
    std::vector<std::thread> th;
    for (unsigned t = 0; t < nth; ++t) {
      th.emplace_back([&, t]() {
        const int ya = y0 + (int)t * chunk_rows;
        const int yb = std::min(N, ya + chunk_rows);
        std::string& out = cur[t];
        out.clear();
        if (ya >= yb) return;
        out.reserve((size_t)(yb - ya) * NN * (expo_data == 1 ? 7 * 20 : 2 * 20));
        char tmp[7 * (F15_MAX + 1)];  // 7 values and their separators
        for (int y = ya; y < yb; ++y)
          for (int x = 0; x < N; ++x)
            for (int z = 0; z < N; ++z) {
              const size_t i = ((size_t)z * N + y) * N + x;
              char* q = tmp;
              if (expo_data == 1) {
                const double v[7] = {u[i], u[n + i], u[2 * n + i], P[i], P[n + i], P[2 * n + i], phi[i]};
                for (int c = 0; c < 7; ++c) {
                  q = put_f15(q, v[c]);
                  *q++ = c < 6 ? ' ' : '\n';
                }
              } else {
                q = put_f15(q, u[i]);
                *q++ = ' ';
                q = put_f15(q, u[n + i]);
                *q++ = ' ';
              }
              out.append(tmp, (size_t)(q - tmp));
            }
      });
    }
    for (auto& t : th) t.join();
    if (writer.joinable()) writer.join();  // round k - 1 written: its buffers may be reused next
    std::vector<std::string>* done = &cur;
    writer = std::thread([done, fp, &err]() {
      for (auto& b : *done)
        if (!b.empty() && std::fwrite(b.data(), 1, b.size(), fp) != b.size()) err = 1;
    });
  }
  if (writer.joinable()) writer.join();
  if (std::fclose(fp) != 0) err = 1;
  if (err) return set_error(TTSH_E_IO, std::string("write failed: ") + path);
  return TTSH_OK;
}

int ttsh_init_reference(const ttsh_input* in, unsigned seed, const char* conf0_path, double* phi, double* P,
                        double* u, double* ustar, double* Pstar) {
  if (!in || !phi || !P || !u || !ustar || !Pstar) return set_error(TTSH_E_INVALID, "ttsh_init_reference: null");
  const int N = in->Nx;
  if (N <= 0 || in->Ny != N || in->Nz != N) return set_error(TTSH_E_INVALID, "ttsh_init_reference: grid");
  const size_t n = (size_t)N * N * N;
  if (in->InitCond != 1) {
    std::fill(phi, phi + n, 0.0);
    std::fill(P, P + 3 * n, 0.0);
    std::fill(u, u + 3 * n, 0.0);
    std::fill(ustar, ustar + 3 * n, 0.0);
    std::fill(Pstar, Pstar + 3 * n, 0.0);
  }
  if (in->InitCond == 0) {  // the two velocity columns of data/conf_<t0>.dat, in the same loop order
    std::ifstream conf;
    if (conf0_path) conf.open(conf0_path);
    for (int i = 0; i < N; i++)
      for (int j = 0; j < N; j++)
        for (int k = 0; k < N; k++) {
          const size_t idx = ((size_t)k * N + j) * N + i;  // x = i, y = j, z = k (TTSH3D.cu:786-791)
          conf >> u[idx] >> u[n + idx];
        }
    return TTSH_OK;
  }
  if (in->InitCond != 1) return TTSH_OK;
  // InitCond 1: 14 draws per site (12 fields, then p_v and p_p, which the first projection
  // recomputes) in the loop order x, y, z (z innermost), from std::default_random_engine(seed)
  // through uniform_real_distribution<double>. That engine is minstd_rand0 (x <- 16807 x mod
  // 2^31 - 1), and each double draw takes two of its outputs (generate_canonical<double, 53> of a
  // 2^31 - 2 wide range), so site s starts at the state x_0 16807^(28 s): the sites are drawn on
  // all host cores with the reference's numbers.
  constexpr uint64_t LCG_A = 16807, LCG_M = 2147483647;
  auto powmod = [](uint64_t b, uint64_t e) {
    uint64_t r = 1;
    for (b %= LCG_M; e; e >>= 1, b = b * b % LCG_M)
      if (e & 1) r = r * b % LCG_M;
    return r;
  };
  const uint64_t x0 = (uint64_t)seed % LCG_M == 0 ? 1 : (uint64_t)seed % LCG_M;  // the engine's seeding rule
  // Work unit: XB consecutive x = i (one 64-byte line of each field along x), one engine per x
  // column started at its first site s = i N^2, the sites then visited in (y, z, x) order so that
  // the writes fill whole lines; units go to the threads round-robin.
  constexpr int XB = 8;
  const int nunits = (N + XB - 1) / XB;
  const unsigned nth = std::max(1u, std::min({64u, std::thread::hardware_concurrency(), (unsigned)nunits}));
  const uint64_t step_col = powmod(LCG_A, 28 * (uint64_t)N * N);  // one x column: N^2 sites
  const uint64_t start0 = x0;
  std::vector<std::thread> th;
  for (unsigned t = 0; t < nth; ++t)
    th.emplace_back([&, t]() {
      for (int unit = (int)t; unit < nunits; unit += (int)nth) {
        const int ia = unit * XB, nb = std::min(XB, N - ia);
        std::default_random_engine rng[XB];
        uint64_t st = start0 * powmod(step_col, (uint64_t)ia) % LCG_M;  // state at site s = ia N^2
        for (int b = 0; b < nb; ++b) {
          rng[b].seed((std::default_random_engine::result_type)st);
          st = st * step_col % LCG_M;
        }
        std::uniform_real_distribution<double> randUR;
        for (int j = 0; j < N; j++)
          for (int k = 0; k < N; k++)
            for (int b = 0; b < nb; ++b) {
              const int i = ia + b;
              const size_t idx = ((size_t)k * N + j) * N + i;  // x = i, y = j, z = k (TTSH3D.cu:786-791)
              double* tgt[12] = {&u[idx], &u[n + idx], &u[2 * n + idx], &ustar[idx], &ustar[n + idx],
                                 &ustar[2 * n + idx], &P[idx], &P[n + idx], &P[2 * n + idx], &Pstar[idx],
                                 &Pstar[n + idx], &Pstar[2 * n + idx]};
              for (int c = 0; c < 12; ++c) *tgt[c] = 0 + in->init0 * (randUR(rng[b]) - 0.5);
              const double dx = (i - in->Nx / 2.), dy = (j - in->Ny / 2.), dz = (k - in->Nz / 2.);
              const double r = std::sqrt(dx * dx + dy * dy + dz * dz);
              phi[idx] = (1 - std::tanh((r - in->Nx / 4.) * 2)) / 2;
              (void)randUR(rng[b]);  // p_v (recomputed by the first projection)
              (void)randUR(rng[b]);  // p_p
            }
      }
    });
  for (auto& x : th) x.join();
  return TTSH_OK;
}

}  // extern "C"

namespace {

inline uint64_t splitmix64(uint64_t x) {
  x += 0x9E3779B97F4A7C15ull;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  return x ^ (x >> 31);
}
// Counter-based uniform in [0,1): stream `k` of site `idx` under `seed`.
inline double uni(uint64_t seed, uint64_t idx, uint64_t k) {
  return (double)(splitmix64(splitmix64(seed) ^ (idx * 8 + k)) >> 11) * (1.0 / 9007199254740992.0);
}

}  // namespace

extern "C" int ttsh_init_droplet(int N, double h, double R, double xi, uint64_t seed, double angular_noise, double* phi,
                                 double* P) {
  if (N < 4 || !(h > 0) || !(xi > 0) || !phi || !P)
    return set_error(TTSH_E_INVALID, "ttsh_init_droplet: bad arguments");
  const size_t n = (size_t)N * N * N;
  const double c = N / 2.0, twopi = 6.283185307179586476925286766559;
  // scratch left uninitialised here: the slabs below write every element (and touch its pages) on
  // the thread that computes it
  std::unique_ptr<double[]> Qb(new double[3 * n]), Tb(new double[3 * n]);
  double* Q = Qb.get();
  double* T2 = Tb.get();
  // Every site is a function of its own index (counter-based draws) and, in the smoothing passes,
  // of the previous pass: z-slabs are computed on all host cores with the same results.
  const unsigned nth = std::max(1u, std::min({64u, std::thread::hardware_concurrency(), (unsigned)N}));
  auto slabs = [&](auto&& body) {
    std::vector<std::thread> th;
    for (unsigned t = 0; t < nth; ++t)
      th.emplace_back([&, t]() {
        const int z0 = (int)((long long)N * t / nth), z1 = (int)((long long)N * (t + 1) / nth);
        body(z0, z1);
      });
    for (auto& t : th) t.join();
  };
  slabs([&](int z0, int z1) {
    for (int z = z0; z < z1; ++z)
      for (int y = 0; y < N; ++y)
        for (int x = 0; x < N; ++x) {
          const size_t i = ((size_t)z * N + y) * N + x;
          const double dx = x - c, dy = y - c, dz = z - c;
          const double r = h * std::sqrt(dx * dx + dy * dy + dz * dz);
          phi[i] = 0.5 * (1.0 - std::tanh((r - R) / xi));
          if (phi[i] > 0.5) {
            const double cz = 1.0 - 2.0 * uni(seed, i, 0);
            const double az = twopi * uni(seed, i, 1);
            const double s = std::sqrt(std::max(0.0, 1.0 - cz * cz));
            double v[3] = {s * std::cos(az), s * std::sin(az), cz};
            if (angular_noise > 0) {
              double g[3];
              for (int k = 0; k < 3; ++k) {  // Box-Muller
                const double u1 = 1.0 - uni(seed, i, 2 + k), u2 = uni(seed, i, 5 + (k % 3));
                g[k] = std::sqrt(-2.0 * std::log(u1)) * std::cos(twopi * u2);
              }
              const double gp = g[0] * v[0] + g[1] * v[1] + g[2] * v[2];
              double w[3], nn = 0;
              for (int k = 0; k < 3; ++k) {
                w[k] = v[k] + angular_noise * (g[k] - gp * v[k]);
                nn += w[k] * w[k];
              }
              nn = std::sqrt(nn);
              for (int k = 0; k < 3; ++k) v[k] = w[k] / nn;
            }
            for (int k = 0; k < 3; ++k) Q[k * n + i] = v[k];
          } else {
            for (int k = 0; k < 3; ++k) Q[k * n + i] = 0.0;
          }
        }
  });
  // 3 Jacobi passes: mean of self and the 6 face neighbours, periodic.
  const size_t NN = (size_t)N * N;
  for (int pass = 0; pass < 3; ++pass) {
    slabs([&](int z0, int z1) {
      for (int k = 0; k < 3; ++k) {
        const double* a = &Q[k * n];
        double* b = &T2[k * n];
        for (int z = z0; z < z1; ++z) {
          const size_t zm = (size_t)(z == 0 ? N - 1 : z - 1) * NN, zc = (size_t)z * NN,
                       zp = (size_t)(z == N - 1 ? 0 : z + 1) * NN;
          for (int y = 0; y < N; ++y) {
            const size_t ym = (size_t)(y == 0 ? N - 1 : y - 1) * N, yc = (size_t)y * N,
                         yp = (size_t)(y == N - 1 ? 0 : y + 1) * N;
            for (int x = 0; x < N; ++x) {
              const int xm = x == 0 ? N - 1 : x - 1, xp = x == N - 1 ? 0 : x + 1;
              b[zc + yc + x] = (a[zc + yc + x] + a[zc + yc + xm] + a[zc + yc + xp] + a[zc + ym + x] +
                                a[zc + yp + x] + a[zm + yc + x] + a[zp + yc + x]) / 7.0;
            }
          }
        }
      }
    });
    std::swap(Q, T2);
  }
  slabs([&](int z0, int z1) {
    for (size_t i = (size_t)z0 * NN; i < (size_t)z1 * NN; ++i)
      for (int k = 0; k < 3; ++k) P[k * n + i] = phi[i] > 0.5 ? Q[k * n + i] : 0.0;
  });
  return TTSH_OK;
}
