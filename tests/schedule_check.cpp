// Host check of the fused kernels' persistent work split (bacterial-droplet_gb300/csrc/schedule.h,
// the code the kernels run): for many grid sizes, droplet counts, plane counts and tile shapes,
// every (droplet, tile, plane) is swept exactly once, and every segment lies in one slab and one
// tile column. Prints "ok" or the first failure.
#include <cstdio>
#include <vector>

#include "schedule.h"

int main() {
  const int Ns[] = {32, 64, 96, 128, 160, 192, 256, 512};
  const int THs[] = {8, 16, 32};
  const int ninsts[] = {1, 2, 3, 7, 24, 64};
  const int Gs[] = {1, 2, 3, 7, 151, 152, 304, 456, 1000, 4096};
  long long configs = 0;
  for (int N : Ns)
    for (int TH : THs)
      for (int ninst : ninsts) {
        if ((long long)ninst * N * N * N > (1ll << 29)) continue;  // keep the check quick
        const int TPI = (N / 32) * (N / TH);
        const long long planes = (long long)ninst * TPI * N;
        for (int G : Gs) {
          if (G > planes) continue;  // the launch caps the grid at the number of planes
          std::vector<unsigned char> seen(planes, 0);
          int S = N;
          while (S > 128 && S % 2 == 0) S /= 2;
          for (int b = 0; b < G; ++b) {
            ttsh::SweepSplit sp(N, TPI, ninst, G, b);
            int inst, t, z0, z1;
            while (sp.next(inst, t, z0, z1)) {
              if (inst < 0 || inst >= ninst || t < 0 || t >= TPI || z0 < 0 || z1 > N || z1 <= z0 ||
                  z0 / S != (z1 - 1) / S) {
                std::printf("bad segment N=%d TH=%d ninst=%d G=%d b=%d: inst %d tile %d z %d..%d\n", N, TH, ninst, G, b,
                            inst, t, z0, z1);
                return 1;
              }
              for (int z = z0; z < z1; ++z) {
                const long long i = ((long long)inst * TPI + t) * N + z;
                if (seen[i]++) {
                  std::printf("site swept twice N=%d TH=%d ninst=%d G=%d: inst %d tile %d z %d\n", N, TH, ninst, G,
                              inst, t, z);
                  return 1;
                }
              }
            }
          }
          for (long long i = 0; i < planes; ++i)
            if (!seen[i]) {
              std::printf("site not swept N=%d TH=%d ninst=%d G=%d: index %lld\n", N, TH, ninst, G, i);
              return 1;
            }
          ++configs;
        }
      }
  std::printf("ok %lld configurations\n", configs);
  return 0;
}
