// schedule.h — the work split of the fused kernels' persistent grid (fused.cu), in a form the
// device code and a host-side check of its coverage share.
//
// The output sites of a group of droplets are cut into items (droplet, slab of S planes, tile),
// S the largest divisor of N reached by halving N while it is above 128. In rounds, CTA b of G
// sweeps items b, b + G, b + 2G, ... while every CTA has a whole item (so the CTAs running at the
// same time hold neighbouring tiles of one slab); the items left over are cut into G equal runs
// of planes, one per CTA (so no SM waits out a partial wave). Each (item, run of planes) is one
// segment: one tile column over planes z0 .. z1 - 1 of one slab.
#pragma once

#ifdef __CUDACC__
#define TTSH_HD __host__ __device__ __forceinline__
#else
#define TTSH_HD inline
#endif

namespace ttsh {

struct SweepSplit {
  int TPI, S, NS, G, b, full, k;
  long long w, w1;

  // N: planes (and columns) of a droplet; tpi: tiles per plane of a droplet; ninst: droplets;
  // G: CTAs of the grid; b: this CTA.
  TTSH_HD SweepSplit(int N, int tpi, int ninst, int G_, int b_) : TPI(tpi), S(N), G(G_), b(b_), k(0) {
    while (S > 128 && S % 2 == 0) S /= 2;
    NS = N / S;
    const int items = ninst * NS * TPI;
    full = items / G;
    const long long rest = (long long)(items - full * G) * S;  // planes of the items left over
    w = (long long)b * rest / G;
    w1 = (long long)(b + 1) * rest / G;
  }

  // The next segment of this CTA: droplet, tile (row-major within a plane) and planes z0 .. z1 - 1;
  // false when the CTA's share is done.
  TTSH_HD bool next(int& inst, int& tile, int& z0, int& z1) {
    int item, za, zb;
    if (k < full) {
      item = k++ * G + b;
      za = 0;
      zb = S;
    } else if (w < w1) {
      const int q = (int)(w / S);
      za = (int)(w - (long long)q * S);
      const long long left = w1 - w;
      zb = (long long)(S - za) < left ? S : (int)(za + left);
      item = full * G + q;
      w += zb - za;
    } else {
      return false;
    }
    inst = item / (NS * TPI);
    const int r = item - inst * NS * TPI;
    const int sl = r / TPI;
    tile = r - sl * TPI;
    z0 = sl * S + za;
    z1 = sl * S + zb;
    return true;
  }
};

}  // namespace ttsh
