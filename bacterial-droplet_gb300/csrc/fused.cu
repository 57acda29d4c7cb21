// fused.cu — the fused FP32 form of the TTSH3D step.
//
// Three kernels replace stage1 + stage2 + div + correct of the plain form (plain.cu):
//
//   fused_rhs     phi, P, u -> u*, P*, phi'   (getTempVari_1/2 + getDtF + getVStar + the phi
//                 update of getVNew, TTSH3D.cu:537-632, :471-491, :515), all intermediates
//                 (mu_0, mu_b, the stress S_ab, D_a P_b) kept on chip.
//   fused_div     u*, P* -> W = div(u*)/dt + i div(P*)/dt   (getStream mode 0, :664-670, with
//                 the reference's stale halo for neighbours across the periodic boundary)
//   fused_correct u*, P*, W -> u, P   (getVNew, :505-511)
//
// u, u* and P* are stored compensated: the FP32 value, which the stencils read, and in bf16 the
// part of the exact value that FP32 rounding dropped, carried through every update (TwoSum); P is
// the FP32 value nearest the exact update.
// The divergence that feeds the pressure is taken exactly from both (fused_div): u* is nearly
// solenoidal, so its divergence is a small difference of large values, and 1/dt amplifies
// whatever rounding it carries into the pressure.
//
// All three march along z through a tile of columns (a "2.5D" sweep; fused_rhs 32 x 8, fused_div
// 32 x 16, fused_correct 32 x 16), on a chunked or a persistent schedule: each z-plane of
// every field the stencils need is staged once in a shared-memory ring of planes, and each
// thread evaluates the 27-point derivatives / 15-point Laplacians of a 1 x R strip of sites
// from its 3 x (R+2) x 3 neighbourhood, so warps read shared memory with unit stride. The
// nested stencils of the RHS (sigma and mu need D P and L P; the velocity update needs D sigma
// and L mu) are staged: stage 1 forms the products of plane z+1 while the thread of each tile
// column finishes plane z. It splits those outer stencils into in-plane partial sums and
// carries the z-combination in registers from plane to plane, so every product plane is read
// once.
//
// fused_rhs computes on pairs of fields ((phi, Px), (Py, Pz), (ux, uy), and pairs of products)
// with the packed FP32 instructions of sm_100+ (add/mul/fma .f32x2, two independent IEEE FP32
// operations with round-to-nearest, the same results as two scalar ones). The state planes are
// staged planar (one array per field, 16-byte copies); the products are stored as float2 pairs,
// so that one 64-bit load fetches both.
//
// The stencil arithmetic is the reference's 27-point and 15-point weights (st_dx/st_dy/st_dz/
// st_lap of common.cuh, TTSH3D.cu:3280-3343) in FP32, regrouped separably; the stress enters as
// one field per component, S_ab = cA phi D_a P_b - zeta phi P_a P_b, whose divergence is the
// reference's cA * div(sigma) plus the build-defined active stress.
#include <algorithm>
#include <cstdio>
#include <stdexcept>
#include <utility>

#include "common.cuh"
#include "kernels.h"
#include "schedule.h"

namespace ttsh {

namespace {

constexpr int TX = 32, TY = 16;   // output tile (columns) of fused_correct
constexpr int TYR = 8;            // fused_rhs: tiles of TX x TYR columns, two CTAs per SM
constexpr int RB = 2;             // strip length (sites per thread) of fused_rhs stage 1 (a 4-row window)
constexpr int NT = TX * TYR;      // threads of fused_rhs: one tile column each in phase 2
constexpr int US = 4;             // strip length of the velocity terms (phase 1)

// fused_rhs regions: A = tile + 2 (phi, P), B = tile + 1 (u, stage-1 products), C = tile.
constexpr int AH = TYR + 4;
constexpr int BW = TX + 2, BH = TYR + 2;
// The staged state planes are planar (one array per field), rows of SXW floats from x0 - 4 to
// x0 + TX + 3, copied in 16-byte chunks (4 sites): a chunk starts at a multiple of 4, so it never
// straddles the periodic boundary and the copies are whole aligned segments. The A ring holds
// (phi, Px, Py, Pz) over rows y0 - 2 .. y0 + TYR + 1, the u ring (ux, uy, uz) over rows
// y0 - 1 .. y0 + TYR. Column of x: x - x0 + 4. Staged row r starts at srow(r): every second row
// is skewed by one more chunk, so that the stage-1 strips of the last two B columns (rows
// 0, 2, .., 8 apart in one warp) read ten different banks; strips start at even rows, so a
// window row's offset from its strip's first row is srow(r) too.
constexpr int SXW = TX + 8, SXC = SXW / 4;
__host__ __device__ constexpr int srow(int r) { return r * SXW + 4 * (r >> 1); }
constexpr int AFP = srow(AH - 1) + SXW;  // floats per field plane, A ring
constexpr int UFP = srow(BH - 1) + SXW;  // floats per field plane, u ring
constexpr int CN = TX * TY;  // fused_correct's tile
// Row pitches of the products, one element longer than the rows: warps whose lanes sit in
// different rows (the stage-1 strips of the last two B columns) then hit different banks.
constexpr int BP = BW + 1, BNP = BP * BH;  // B region
constexpr int CP = TX + 1, CNP = CP * TYR;  // the tile (partials)
// Products of one plane on B, as float2 pairs (plus one scalar field):
//   M0 = (mu_0, mu_x), M1 = (mu_y, mu_z)       Laplacians: phi', P*
//   T0 = (S_xy, S_xz), T1 = (S_yy, S_yz), T2 = (S_zy, S_zz)   divergence columns y, z
//   T3 = (S_xx, S_yx), and S_zx alone                          divergence column x
constexpr int PM0 = 0, PM1 = 1, PT0 = 2, PT1 = 3, PT2 = 4, PT3 = 5, NPR = 6;
// Pointwise parts of the update on C ("partials"), float2 pairs:
//   Q0 = (u_x, u_y) terms, Q1 = (u_z term, phi term), Q2 = (P_x, P_y) terms, Q3 = (P_z term, -)
constexpr int NPQ = 4;
// Shared memory (bytes): A ring RA planes x 4 fields; u ring RU planes x 3 fields; one plane of
// products; partials ring 2 planes. The A and u rings hold one plane more than the stencils
// read: the next plane is copied into it (cp.async) while the current ones compute.
constexpr int RA = 4, RU = 4;
constexpr size_t OFF_A = 0;
constexpr size_t OFF_U = OFF_A + (size_t)RA * 4 * AFP * sizeof(float);
constexpr size_t OFF_PR = OFF_U + (size_t)RU * 3 * UFP * sizeof(float);
constexpr size_t OFF_SZX = OFF_PR + (size_t)NPR * BNP * sizeof(float2);
constexpr size_t OFF_PQ = OFF_SZX + (((size_t)BNP * sizeof(float) + 15) / 16) * 16;
constexpr size_t RHS_SMEM = OFF_PQ + (size_t)2 * NPQ * CNP * sizeof(float2);
static_assert(2 * RHS_SMEM <= 227 * 1024, "fused_rhs: two CTAs per SM");
static_assert(OFF_U % 16 == 0 && OFF_PR % 16 == 0 && OFF_SZX % 16 == 0 && OFF_PQ % 16 == 0 &&
                  (AFP * sizeof(float)) % 16 == 0 && (UFP * sizeof(float)) % 16 == 0 && (SXW * sizeof(float)) % 16 == 0,
              "16-byte aligned regions, field planes and rows");
// copy roles: (row, chunk) items of the A region, then of the u region, one thread each
constexpr int NIA = AH * SXC, NIU = BH * SXC;
static_assert(NIA + NIU <= NT, "one staged (row, chunk) item per thread");
// phase-1 thread roles of fused_rhs: stage-1 strips of the B region, then the velocity strips
constexpr int NS1 = (BW * BH) / RB;                   // 204 stage-1 strips
constexpr int NU0 = ((NS1 + 31) / 32) * 32;           // first velocity thread (warp aligned)
constexpr int NUS = TX * (TYR / US);                  // velocity strips
static_assert((BH % RB) == 0 && (TYR % US) == 0, "strip lengths divide the regions");
static_assert(NU0 + NUS <= NT, "phase-1 roles fit the block");

__device__ __forceinline__ int wrapN(int a, int N) { return a < 0 ? a + N : (a >= N ? a - N : a); }

// Asynchronous global -> shared copies (cp.async): the data lands while the CTA computes.
__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;\n" ::: "memory"); }

// Arithmetic on one value (float) or a pair (float2, packed FP32).
__device__ __forceinline__ float vadd(float a, float b) { return a + b; }
__device__ __forceinline__ float vsub(float a, float b) { return a - b; }
__device__ __forceinline__ float vmul(float a, float b) { return a * b; }
__device__ __forceinline__ float vfma(float a, float b, float c) { return fmaf(a, b, c); }
__device__ __forceinline__ float vsplat(float a, float) { return a; }
__device__ __forceinline__ float2 vadd(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 vsub(float2 a, float2 b) {
  float2 d;
  asm("sub.rn.f32x2 %0, %1, %2;"
      : "=l"(*reinterpret_cast<unsigned long long*>(&d))
      : "l"(*reinterpret_cast<const unsigned long long*>(&a)), "l"(*reinterpret_cast<const unsigned long long*>(&b)));
  return d;
}
__device__ __forceinline__ float2 vmul(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 vfma(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ float2 vsplat(float a, float2) { return make_float2(a, a); }
__device__ __forceinline__ float2 f2(float a, float b) { return make_float2(a, b); }

// Separable evaluation (FP32). With s = [1, 4, 1] and delta = [-1, 0, 1]:
//   D_x = c2h/36 * delta_x s_y s_z,  D_y = c2h/36 * s_x delta_y s_z,  D_z = c2h/36 * s_x s_y delta_z,
//   L = cl12 * (8 corners - 8 centre) + cl23 * (6 faces - 6 centre)  (corners = c_x c_y c_z,
//       c = [1, 0, 1]),
// the reference's 27-point and 15-point weights (TTSH3D.cu:3280-3343) regrouped. Each row of the
// neighbourhood (3 planes x 3 columns) is reduced to the few sums the R sites of the strip share.
// The Laplacian is written shift-invariant: the reference's -14/(3h^2) centre weight is split
// between the two neighbour sums (8 cl12 + 6 cl23 = 14/(3h^2)), each of which subtracts the centre
// before its weight is applied, so that a constant field has exactly zero Laplacian in FP32. With
// the three weights rounded to FP32 separately, L(1) would be about 2.4e-7/h^2 instead of zero: a
// systematic term, e.g. a spurious -kPhi 2.4e-7 phi in mu_0, whose force mu_0 D phi is a gradient
// that the pressure absorbs as a smooth error.
struct SepK {
  float d;  // c2h / 36
  float l12, l23, l143;
  float lz;  // 1/h^2 = 4 l12 + l23 (the z-carried form's weight of the centre column)
};
// ld(z, r, c): the value at plane z (0..2 = offset -1..1), strip row r (0..R+1 = offset -1..R),
// column c (0..2 = offset -1..1). ctr[i] receives the centre value of site i.
template <int R, bool DX, bool DY, bool DZ, bool LAP, class V, class LD>
__device__ __forceinline__ void sep_rows(const LD& ld, const SepK& k, V* dx, V* dy, V* dz, V* lap, V* ctr) {
  const V four = vsplat(4.f, V()), kd = vsplat(k.d, V());
  V a[R + 2], b[R + 2], c[R + 2], e[R + 2], f[R + 2], g[R + 2], h[R + 2];
#pragma unroll
  for (int r = 0; r < R + 2; ++r) {
    V v0[3], v1[3], v2[3], cz[3], sz[3], dzr[3];
#pragma unroll
    for (int q = 0; q < 3; ++q) {
      v0[q] = ld(0, r, q);
      v1[q] = ld(1, r, q);
      v2[q] = ld(2, r, q);
      cz[q] = vadd(v0[q], v2[q]);
      sz[q] = vfma(four, v1[q], cz[q]);
      dzr[q] = vsub(v2[q], v0[q]);
    }
    a[r] = vsub(sz[2], sz[0]);                       // delta_x of s_z
    b[r] = vfma(four, sz[1], vadd(sz[0], sz[2]));    // s_x of s_z
    c[r] = vfma(four, dzr[1], vadd(dzr[0], dzr[2])); // s_x of delta_z
    e[r] = vadd(cz[0], cz[2]);                       // corners of the row
    f[r] = cz[1];                                    // z faces
    g[r] = vadd(v1[0], v1[2]);                       // x faces
    h[r] = v1[1];                                    // centre column of the centre plane
  }
#pragma unroll
  for (int i = 0; i < R; ++i) {
    if (DX) dx[i] = vmul(kd, vfma(four, a[i + 1], vadd(a[i], a[i + 2])));
    if (DY) dy[i] = vmul(kd, vsub(b[i + 2], b[i]));
    if (DZ) dz[i] = vmul(kd, vfma(four, c[i + 1], vadd(c[i], c[i + 2])));
    if (LAP) {
      const V c = h[i + 1];
      const V corners = vadd(e[i], e[i + 2]);
      const V faces = vadd(vadd(f[i + 1], g[i + 1]), vadd(h[i], h[i + 2]));
      // corners - 8c: 8c is exact; faces - 6c with 6c rounded as the sum of the faces is, so that
      // both differences vanish exactly for a constant field
      lap[i] = vfma(vsplat(k.l12, V()), vfma(vsplat(-8.f, V()), c, corners),
                    vmul(vsplat(k.l23, V()), vsub(faces, vmul(vsplat(6.f, V()), c))));
    }
    if (ctr) ctr[i] = h[i + 1];
  }
}

// s + e = a + b exactly (Knuth's TwoSum: six FP32 additions, no assumption on the magnitudes).
__device__ __forceinline__ float two_sum(float a, float b, float& e) {
  const float s = a + b;
  const float bb = s - a;
  e = (a - (s - bb)) + (b - bb);
  return s;
}

// x* = x + d stored compensated: the FP32 sum and, in bf16, what its rounding dropped plus the
// compensation x_lo that x brought along. Returns the FP32 value.
// `stride` 2 for one half of the pairs star / starlo.
__device__ __forceinline__ float put_comp(float* hi, __nv_bfloat16* lo, size_t g, float x, float d, __nv_bfloat16 x_lo,
                                          int stride = 1) {
  float e;
  const float s = two_sum(x, d, e);
  hi[stride * g] = s;
  lo[stride * g] = __float2bfloat16_rn(e + __bfloat162float(x_lo));
  return s;
}

// ------------------------------------------------------------------------------------------
// One segment of the sweep: the tile column (x0, y0) of droplet I, output planes z0 .. z1 - 1.
__device__ __forceinline__ void rhs_segment(const InstDev<float>& I, int par, int N, int x0, int y0, int z0, int z1,
                                            unsigned char* smr) {
  const Phys<float> p = I.ph;  // by value: read once, kept in registers
  const SepK sk{p.c2h * (1.f / 36.f), p.cl12, p.cl23, p.cl143, p.clz};
  const size_t NN = (size_t)N * N;
  const float* __restrict__ gphi = I.phi[par];
  const float* __restrict__ gP[3] = {I.P[0], I.P[1], I.P[2]};
  const float* __restrict__ gU[3] = {I.U[0], I.U[1], I.U[2]};
  // u*_b and P*_b: the two halves of the pairs star[b] (and of their compensations starlo[b])
  float* oUs[3];
  float* oPs[3];
  __nv_bfloat16* oSlo[6];
#pragma unroll
  for (int b = 0; b < 3; ++b) {
    oUs[b] = reinterpret_cast<float*>(I.star[par ^ 1][b]);
    oPs[b] = oUs[b] + 1;
    oSlo[b] = reinterpret_cast<__nv_bfloat16*>(I.starlo[par ^ 1][b]);
    oSlo[3 + b] = oSlo[b] + 1;
  }
  float amu = 0.f, amp = 0.f;  // max |u*|, |P*| of this thread's outputs (the divergence's grid)
  float* const ophi = I.phi[par ^ 1];
  float* const phic = I.phic;
  float* const sA = reinterpret_cast<float*>(smr + OFF_A);        // [RA][4][AFP]: phi, Px, Py, Pz
  float* const sU = reinterpret_cast<float*>(smr + OFF_U);        // [RU][3][UFP]: ux, uy, uz
  float2* const sPr = reinterpret_cast<float2*>(smr + OFF_PR);    // [NPR][BNP]
  float* const sSzx = reinterpret_cast<float*>(smr + OFF_SZX);    // [BNP]
  float2* const sQ = reinterpret_cast<float2*>(smr + OFF_PQ);     // [2][NPQ][CNP]
  const int tid = threadIdx.x;
  const int niter = (z1 - z0) + 4;

  // issue(i): A plane a = z0 - 2 + i (phi, P over tile+2) into A slot i % RA, and u plane a - 1
  // (tile+1) into u slot i % RU. Iteration i runs stage 1 at plane b = a - 1 and finishes plane
  // c = a - 2; issue(i + 1) runs during iteration i.
  // Thread tid < NIA copies (row, chunk) item tid of the A region for its 4 fields, thread
  // NIA <= tid < NIA + NIU item tid - NIA of the u region for its 3; the offsets within a plane
  // (periodic wrap included) are the same for every plane.
  const bool cpA = tid < NIA, cpU = !cpA && tid < NIA + NIU;
  int goff = 0, soff = 0;
  if (cpA || cpU) {
    const int t = cpA ? tid : tid - NIA;
    const int row = t / SXC, ch = t - row * SXC;
    goff = wrapN((cpA ? y0 - 2 : y0 - 1) + row, N) * N + wrapN(x0 - 4 + 4 * ch, N);
    soff = srow(row) + 4 * ch;
  }
  auto issue = [&](int i) {
    if (cpA) {
      const size_t d = (size_t)wrapN(z0 - 2 + i, N) * NN + goff;
      float* dst = sA + (i % RA) * 4 * AFP + soff;
      cp_async16(dst, gphi + d);
      cp_async16(dst + AFP, gP[0] + d);
      cp_async16(dst + 2 * AFP, gP[1] + d);
      cp_async16(dst + 3 * AFP, gP[2] + d);
    } else if (cpU) {
      const size_t d = (size_t)wrapN(z0 - 3 + i, N) * NN + goff;
      float* dst = sU + (i % RU) * 3 * UFP + soff;
      cp_async16(dst, gU[0] + d);
      cp_async16(dst + UFP, gU[1] + d);
      cp_async16(dst + 2 * UFP, gU[2] + d);
    }
    cp_async_commit();
  };
  // phase 2: thread tid takes the 2-site strip s = tid % 256 of the tile (column px, rows py0,
  // py0 + 1) for one half of the outer stencils: half A (tid < 256) the Laplacians of (mu_0, mu_x),
  // (mu_y, mu_z) and the divergence of stress column x, then P*, phi' and u*_x; half B the
  // divergence of stress columns (y, z), then u*_y, u*_z. Each half has every input of what it
  // writes. The sites' rows share a 4 x 3 window of each product plane.
  static_assert(NT == 2 * TX * (TYR / 2), "phase 2: two halves of 2-site strips");
  const bool halfA = tid < NT / 2;
  const int ps = tid & (NT / 2 - 1);
  const int px = ps % TX, py0 = (ps / TX) * 2;
  const int pbase = py0 * BP + px;  // B index of window row 0 (site 0's row - 1), column px - 1 + 1 - 1
  // z-combinations carried from plane to plane: for a Laplacian, the partial sum of the plane
  // just finished + 1 and that of the plane after it (rL1, rL2); likewise for the divergences.
  // Half A: cv2[0..3] = rL1 [site][pair], cv2[4..7] = rL2, cv1[0..1] = rX1 [site], cv1[2..3] = rX2;
  // half B: cv2[0..1] = rD1 [site], cv2[2..3] = rD2.
  float2 cv2[8];
  float cv1[4];
#pragma unroll
  for (int k = 0; k < 8; ++k) cv2[k] = f2(0.f, 0.f);
#pragma unroll
  for (int k = 0; k < 4; ++k) cv1[k] = 0.f;
  issue(0);
  for (int i = 0; i < niter; ++i) {
    cp_async_wait_all();
    __syncthreads();
    if (i + 1 < niter) issue(i + 1);
    // the compensations of this iteration's output sites (phi, u_x and P in half A; u_y, u_z in
    // half B), loaded before phase 1 so that the phase-1 work covers the loads
    float cprev[2] = {0.f, 0.f};
    __nv_bfloat16 lprev[2][4];
    if (i >= 4) {
#pragma unroll
      for (int k = 0; k < 2; ++k) {
        const size_t g = (size_t)(z0 - 4 + i) * NN + (size_t)(y0 + py0 + k) * N + (x0 + px);
        if (halfA) {
          cprev[k] = phic[g];
          lprev[k][0] = I.lo[0][g];
          lprev[k][1] = lprev[k][2] = lprev[k][3] = __float2bfloat16_rn(0.f);  // P: FP32 state
        } else {
          lprev[k][0] = I.lo[1][g];
          lprev[k][1] = I.lo[2][g];
        }
      }
    }
    // ---- phase 1a, stage 1 at plane b = z0 - 3 + i over B (tile+1): the products mu_0, mu_b,
    //      S_ab that phase 2 differentiates, and on the tile the pointwise parts of the update
    if (i >= 2 && tid < NS1) {
      const float* a0 = sA + ((i + RA - 2) % RA) * 4 * AFP;  // plane b-1
      const float* a1 = sA + ((i + RA - 1) % RA) * 4 * AFP;  // plane b
      const float* a2 = sA + (i % RA) * 4 * AFP;             // plane b+1
      // strips of the B region: warps take 32 consecutive columns of one strip row (unit-stride
      // shared-memory access); the last BW - 32 columns of every row come after them
      constexpr int NSR = BH / RB, NMAIN = 32 * NSR;
      const int s = tid;
      int bx, by0;
      if (s < NMAIN) { bx = s & 31; by0 = (s >> 5) * RB; }
      else { const int e = s - NMAIN; bx = 32 + e % (BW - 32); by0 = (e / (BW - 32)) * RB; }
      // A index of row offset -1, column offset -1 of site 0 (B column bx is x = x0 - 1 + bx)
      const int base = srow(by0) + bx + 2;
      // pair 0 = (phi, Px), pair 1 = (Py, Pz): D_a (3), L and the centre value of each site
      float2 D0[3][RB], L0[RB], C0[RB], D1[3][RB], L1[RB], C1[RB];
      {
        auto ld = [&](int z, int r, int c) {
          const float* pl = (z == 0 ? a0 : (z == 1 ? a1 : a2)) + base + srow(r) + c;
          return f2(pl[0], pl[AFP]);
        };
        sep_rows<RB, true, true, true, true, float2>(ld, sk, D0[0], D0[1], D0[2], L0, C0);
      }
      {
        auto ld = [&](int z, int r, int c) {
          const float* pl = (z == 0 ? a0 : (z == 1 ? a1 : a2)) + base + srow(r) + c;
          return f2(pl[2 * AFP], pl[3 * AFP]);
        };
        sep_rows<RB, true, true, true, true, float2>(ld, sk, D1[0], D1[1], D1[2], L1, C1);
      }
      const float* ub = sU + (i % RU) * 3 * UFP;  // u at plane b
      float2* pq = sQ + (i & 1) * NPQ * CNP;
#pragma unroll
      for (int k = 0; k < RB; ++k) {
        const int o = (by0 + k) * BP + bx;
        const float ph = C0[k].x, px = C0[k].y, py = C1[k].x, pz = C1[k].y;
        // mu_0 = aPhi 2(phi - 3phi^2 + 2phi^3) - kPhi L phi (:567), mu_b = phi P_b + La^2 L P_b (:571-573)
        // 2 aPhi (phi - 3 phi^2 + 2 phi^3) factored as 2 aPhi phi (1 - phi)(1 - 2 phi): for phi near 0
        // or 1 (inside and outside the droplet) the reference's expanded form cancels to a small
        // value that FP32 would resolve only to about 1e-7
        const float poly = p.aPhi2 * (ph * ((1.f - ph) * (1.f - 2.f * ph)));
        const float2 M0 = vfma(f2(-p.kPhi, p.La2), L0[k], f2(poly, ph * px));
        const float2 M1 = vfma(vsplat(p.La2, float2()), L1[k], vmul(vsplat(ph, float2()), C1[k]));
        sPr[PM0 * BNP + o] = M0;
        sPr[PM1 * BNP + o] = M1;
        // S_ab = cA phi D_a P_b - zeta phi P_a P_b (:587-595 and the active stress)
        const float cph = p.cA * ph, zph = p.zeta * ph;
        const float Pa[3] = {px, py, pz};
        float sx[3];
#pragma unroll
        for (int a = 0; a < 3; ++a) {
          sPr[(PT0 + a) * BNP + o] = vfma(vsplat(cph, float2()), D1[a][k], vmul(vsplat(-zph * Pa[a], float2()), C1[k]));
          sx[a] = fmaf(cph, D0[a][k].y, -zph * Pa[a] * px);
        }
        sPr[PT3 * BNP + o] = f2(sx[0], sx[1]);
        sSzx[o] = sx[2];
        const int cx = bx - 1, cy = by0 + k - 1;
        if (cx >= 0 && cx < TX && cy >= 0 && cy < TYR) {
          // pointwise parts of getDtF (:617-631) at this site of plane b:
          //   u_b:  mu_0 D_b phi;  phi: -u.D phi;
          //   P_b:  -(u + lambda0 P).D P_b - P_b (alpha phi + beta |P|^2 + A |D phi|^2 |P|^2)
          //         - A |P| (D phi . P) D_b phi
          const int c = cy * CP + cx;
          const int ou = srow(by0 + k) + bx + 3;
          const float vx = ub[ou], vy = ub[UFP + ou], vz = ub[2 * UFP + ou];
          const float mu0 = M0.x;
          const float gx = D0[0][k].x, gy = D0[1][k].x, gz = D0[2][k].x;  // D phi
          const float P2 = px * px + py * py + pz * pz;
          const float G2 = gx * gx + gy * gy + gz * gz;
          const float GP = gx * px + gy * py + gz * pz;
          const float kap = p.alpha * ph + P2 * (p.beta + p.A * G2);
          const float m = p.A * sqrtf(P2) * GP;
          const float wx = fmaf(p.lambda0, px, vx), wy = fmaf(p.lambda0, py, vy), wz = fmaf(p.lambda0, pz, vz);
          pq[0 * CNP + c] = f2(mu0 * gx, mu0 * gy);
          pq[1 * CNP + c] = f2(mu0 * gz, -(vx * gx + vy * gy + vz * gz));
          const float ppx = -(wx * D0[0][k].y + wy * D0[1][k].y + wz * D0[2][k].y) - kap * px - m * gx;
          float2 t = vmul(vsplat(wx, float2()), D1[0][k]);
          t = vfma(vsplat(wy, float2()), D1[1][k], t);
          t = vfma(vsplat(wz, float2()), D1[2][k], t);
          t = vfma(vsplat(kap, float2()), C1[k], t);
          t = vfma(vsplat(m, float2()), f2(gy, gz), t);
          pq[2 * CNP + c] = f2(ppx, -t.x);
          pq[3 * CNP + c] = f2(-t.y, 0.f);
        }
      }
    }
    // ---- phase 1b, on the threads stage 1 leaves free: the velocity terms of plane c = b - 1,
    //      -u.D u_b + mu L u_b (:617-621), added to that plane's partials (written by stage 1 at
    //      iteration i - 1), for a strip of US sites of one tile column
    if (i >= 4 && tid >= NU0 && tid < NU0 + NUS) {
      const int s = tid - NU0;
      const int vx = s & 31, vy0 = (s >> 5) * US;  // tile coordinates of the strip
      const int sl0 = (i + RU - 2) % RU, sl1 = (i + RU - 1) % RU, sl2 = i % RU;  // planes c-1, c, c+1
      const int base = srow(vy0) + vx + 3;  // u index of row offset -1, column offset -1 of site 0
      float2 Dp[3][US], Lp[US], Cp[US];
      float Dz[3][US], Lz[US], Cz[US];
      {
        auto ld = [&](int z, int r, int c) {
          const int sl = z == 0 ? sl0 : (z == 1 ? sl1 : sl2);
          const float* pl = sU + sl * 3 * UFP + base + srow(r) + c;
          return f2(pl[0], pl[UFP]);
        };
        sep_rows<US, true, true, true, true, float2>(ld, sk, Dp[0], Dp[1], Dp[2], Lp, Cp);
      }
      {
        auto ld = [&](int z, int r, int c) {
          const int sl = z == 0 ? sl0 : (z == 1 ? sl1 : sl2);
          return sU[sl * 3 * UFP + 2 * UFP + base + srow(r) + c];
        };
        sep_rows<US, true, true, true, true, float>(ld, sk, Dz[0], Dz[1], Dz[2], Lz, Cz);
      }
      float2* pq = sQ + ((i + 1) & 1) * NPQ * CNP;
#pragma unroll
      for (int k = 0; k < US; ++k) {
        const int c = (vy0 + k) * CP + vx;
        const float ux = Cp[k].x, uy = Cp[k].y, uz = Cz[k];
        float2 t = vmul(vsplat(-ux, float2()), Dp[0][k]);
        t = vfma(vsplat(-uy, float2()), Dp[1][k], t);
        t = vfma(vsplat(-uz, float2()), Dp[2][k], t);
        t = vfma(vsplat(p.mu, float2()), Lp[k], t);
        const float tz = fmaf(p.mu, Lz[k], -(ux * Dz[0][k] + uy * Dz[1][k] + uz * Dz[2][k]));
        pq[0 * CNP + c] = vadd(pq[0 * CNP + c], t);
        pq[1 * CNP + c].x += tz;
      }
    }
    __syncthreads();
    // ---- phase 2: the in-plane partial sums of the outer stencils over the products of plane
    //      b, carried in z; plane c = b - 1 is then complete
    if (i >= 2) {
      const int zc = z0 - 4 + i;
      const float2* pq = sQ + ((i + 1) & 1) * NPQ * CNP;    // plane c: stage 1 + velocity terms
      const float* uc = sU + ((i + RU - 1) % RU) * 3 * UFP;  // u at plane c
      const float* ac = sA + ((i + RA - 2) % RA) * 4 * AFP;  // phi, P at plane c
      const float2 four = f2(4.f, 4.f);
      if (halfA) {
        float2 lm[2][2];  // [site]: (L mu_0, L mu_x), (L mu_y, L mu_z)
#pragma unroll
        for (int q = 0; q < 2; ++q) {
          const float2* F = sPr + (PM0 + q) * BNP + pbase;
          float2 v[4][3];
#pragma unroll
          for (int r = 0; r < 4; ++r)
#pragma unroll
            for (int c = 0; c < 3; ++c) v[r][c] = F[r * BP + c];
#pragma unroll
          for (int k = 0; k < 2; ++k) {
            // shift-invariant in-plane sums (see SepK): an off-centre plane adds
            // G = l12 (4 diagonals - 4 centre) + lz centre, the centre plane
            // H = l23 (4 edges - 4 centre) - 2 lz centre; G + H + G = L, zero for a constant field
            const float2 ce = v[k + 1][1];
            const float2 dg = vadd(vadd(v[k][0], v[k][2]), vadd(v[k + 2][0], v[k + 2][2]));
            const float2 ed = vadd(vadd(v[k][1], v[k + 2][1]), vadd(v[k + 1][0], v[k + 1][2]));
            const float2 four_c = vmul(four, ce);
            const float2 G = vfma(vsplat(sk.l12, float2()), vsub(dg, four_c), vmul(vsplat(sk.lz, float2()), ce));
            const float2 H = vfma(vsplat(sk.l23, float2()), vsub(ed, four_c), vmul(vsplat(-2.f * sk.lz, float2()), ce));
            lm[k][q] = vadd(cv2[k * 2 + q], G);
            cv2[k * 2 + q] = vadd(cv2[4 + k * 2 + q], H);
            cv2[4 + k * 2 + q] = G;
          }
        }
        // divergence column x: X of S_xx (T3.x), Y of S_yx (T3.y), Z of S_zx
        float dvx[2];
        {
          const float2* T = sPr + PT3 * BNP + pbase;
          const float* Zs = sSzx + pbase;
          float2 t[4][3];
          float z[4][3];
#pragma unroll
          for (int r = 0; r < 4; ++r)
#pragma unroll
            for (int c = 0; c < 3; ++c) {
              t[r][c] = T[r * BP + c];
              z[r][c] = Zs[r * BP + c];
            }
#pragma unroll
          for (int k = 0; k < 2; ++k) {
            // differences first, then the weighted sum of the (small) differences
            const float xd0 = t[k][2].x - t[k][0].x, xd1 = t[k + 1][2].x - t[k + 1][0].x, xd2 = t[k + 2][2].x - t[k + 2][0].x;
            const float xr = fmaf(4.f, xd1, xd0 + xd2);
            const float yr = fmaf(4.f, t[k + 2][1].y - t[k][1].y,
                                  (t[k + 2][0].y - t[k][0].y) + (t[k + 2][2].y - t[k][2].y));
            const float z0c = fmaf(4.f, z[k + 1][0], z[k][0] + z[k + 2][0]);
            const float z1c = fmaf(4.f, z[k + 1][1], z[k][1] + z[k + 2][1]);
            const float z2c = fmaf(4.f, z[k + 1][2], z[k][2] + z[k + 2][2]);
            const float zr = fmaf(4.f, z1c, z0c + z2c);
            const float Qx = xr + yr;
            dvx[k] = cv1[k] + Qx + zr;
            cv1[k] = fmaf(4.f, Qx, cv1[2 + k]);
            cv1[2 + k] = Qx - zr;
          }
        }
        if (i >= 4) {
#pragma unroll
          for (int k = 0; k < 2; ++k) {
            const int c = (py0 + k) * CP + px, oa = srow(py0 + k + 2) + (px + 4), ou = srow(py0 + k + 1) + (px + 4);
            const size_t g = (size_t)zc * NN + (size_t)(y0 + py0 + k) * N + (x0 + px);
            const float2 q0 = pq[0 * CNP + c], q1 = pq[1 * CNP + c], q2 = pq[2 * CNP + c], q3 = pq[3 * CNP + c];
            const float2 A0 = f2(ac[oa], ac[AFP + oa]), A1 = f2(ac[2 * AFP + oa], ac[3 * AFP + oa]);
            // u*_x = u_x + dt d/dt u_x (:480-482)
            const float usx = put_comp(oUs[0], oSlo[0], g, uc[ou], p.dt * fmaf(sk.d, dvx[k], q0.x),
                                       lprev[k][0], 2);
            // P*_b = P_b + dt (pointwise part + eta L mu_b) (:623-629, :486-488)
            const float psx = put_comp(oPs[0], oSlo[3], g, A0.y, p.dt * fmaf(p.eta, lm[k][0].y, q2.x), lprev[k][1], 2);
            const float2 dp2 = vmul(vsplat(p.dt, float2()), vfma(vsplat(p.eta, float2()), lm[k][1], f2(q2.y, q3.x)));
            const float psy = put_comp(oPs[1], oSlo[4], g, A1.x, dp2.x, lprev[k][2], 2);
            const float psz = put_comp(oPs[2], oSlo[5], g, A1.y, dp2.y, lprev[k][3], 2);
            amu = fmaxf(amu, fabsf(usx));
            amp = fmaxf(amp, fmaxf(fabsf(psx), fmaxf(fabsf(psy), fabsf(psz))));
            // phi' = phi + dt (-u.D phi + gamma L mu_0) (:631, :515), compensated: the part of
            // the increment that rounding drops from phi is carried to the next step (otherwise
            // increments below half an ulp of phi are lost, a systematic mass drift)
            const float ph = A0.x;
            const float inc = fmaf(p.dt, fmaf(p.gamma, lm[k][0].x, q1.y), cprev[k]);
            const float nv = ph + inc;
            phic[g] = inc - (nv - ph);
            ophi[g] = nv;
          }
        }
      } else {
        // divergence columns (y, z), packed: X of T0 = (S_xy, S_xz), Y of T1 = (S_yy, S_yz),
        // Z of T2 = (S_zy, S_zz)
        float2 dv[2];
        {
          const float2* X = sPr + PT0 * BNP + pbase;
          const float2* Y = sPr + PT1 * BNP + pbase;
          const float2* Z = sPr + PT2 * BNP + pbase;
          float2 xa[4][2], ya[4][3], za[4][3];
#pragma unroll
          for (int r = 0; r < 4; ++r) {
            xa[r][0] = X[r * BP];
            xa[r][1] = X[r * BP + 2];
#pragma unroll
            for (int c = 0; c < 3; ++c) {
              ya[r][c] = Y[r * BP + c];
              za[r][c] = Z[r * BP + c];
            }
          }
#pragma unroll
          for (int k = 0; k < 2; ++k) {
            // differences first, then the weighted sum of the (small) differences
            const float2 xr = vfma(four, vsub(xa[k + 1][1], xa[k + 1][0]),
                                   vadd(vsub(xa[k][1], xa[k][0]), vsub(xa[k + 2][1], xa[k + 2][0])));
            const float2 yr = vfma(four, vsub(ya[k + 2][1], ya[k][1]),
                                   vadd(vsub(ya[k + 2][0], ya[k][0]), vsub(ya[k + 2][2], ya[k][2])));
            const float2 t0 = vfma(four, za[k + 1][0], vadd(za[k][0], za[k + 2][0]));
            const float2 t1 = vfma(four, za[k + 1][1], vadd(za[k][1], za[k + 2][1]));
            const float2 t2 = vfma(four, za[k + 1][2], vadd(za[k][2], za[k + 2][2]));
            const float2 zr = vfma(four, t1, vadd(t0, t2));
            const float2 Q = vadd(xr, yr);
            dv[k] = vadd(vadd(cv2[k], Q), zr);
            cv2[k] = vfma(four, Q, cv2[2 + k]);
            cv2[2 + k] = vsub(Q, zr);
          }
        }
        if (i >= 4) {
#pragma unroll
          for (int k = 0; k < 2; ++k) {
            const int c = (py0 + k) * CP + px, ou = srow(py0 + k + 1) + (px + 4);
            const size_t g = (size_t)zc * NN + (size_t)(y0 + py0 + k) * N + (x0 + px);
            const float2 q0 = pq[0 * CNP + c], q1 = pq[1 * CNP + c];
            // (u*_y, u*_z) = (u_y, u_z) + dt d/dt (u_y, u_z) (:480-482)
            const float2 du = vmul(vsplat(p.dt, float2()), vfma(vsplat(sk.d, float2()), dv[k], f2(q0.y, q1.x)));
            const float usy = put_comp(oUs[1], oSlo[1], g, uc[UFP + ou], du.x, lprev[k][0], 2);
            const float usz = put_comp(oUs[2], oSlo[2], g, uc[2 * UFP + ou], du.y, lprev[k][1], 2);
            amu = fmaxf(amu, fmaxf(fabsf(usy), fabsf(usz)));
          }
        }
      }
    }
  }
  record_wmax(I.smax, amu, amp);
}

// The two schedules of the three fused kernels. zc > 0: CTA (bx, by, bz) sweeps tile (bx, by)
// (TW x TH columns) of droplet bz / nchunk over the zc planes of chunk bz % nchunk. zc == 0: a
// persistent grid (as many CTAs as fit on the device at once) splits the group's sites as
// SweepSplit (schedule.h) says. seg(inst, x0, y0, z0, z1) sweeps one segment. Each kernel is
// built for both (PERSIST), so that the chunked form carries no loop state.
template <int TW, int TH, bool PERSIST, class F>
__device__ __forceinline__ void sweep_schedule(int N, int nchunk, int zc, int ninst, F&& seg) {
  if constexpr (!PERSIST) {
    const int z0 = (blockIdx.z % nchunk) * zc;
    seg((int)(blockIdx.z / nchunk), (int)blockIdx.x * TW, (int)blockIdx.y * TH, z0, min(z0 + zc, N));
    return;
  }
  const int TXN = N / TW;  // tile columns per row
  SweepSplit split(N, TXN * (N / TH), ninst, (int)gridDim.x, (int)blockIdx.x);
  int inst, t, z0, z1;
  while (split.next(inst, t, z0, z1)) {  // one call site of seg
    seg(inst, (t % TXN) * TW, (t / TXN) * TH, z0, z1);
    __syncthreads();  // the next segment refills the rings the last one read
  }
}

template <bool PERSIST>
__global__ void __launch_bounds__(NT, 2) k_fused_rhs(const InstDev<float>* __restrict__ insts, int par, int nchunk, int zc,
                                                     int ninst) {
  extern __shared__ __align__(16) unsigned char smr[];
  const int N = insts[0].N;
  // this step's maxima of the Poisson source start from zero (fused_div records them)
  if (blockIdx.x == 0 && blockIdx.y == 0 && blockIdx.z == 0)
    for (int i = threadIdx.x; i < 2 * ninst; i += blockDim.x) insts[i >> 1].wmax[i & 1] = 0;
  sweep_schedule<TX, TYR, PERSIST>(N, nchunk, zc, ninst, [&](int inst, int x0, int y0, int z0, int z1) {
    rhs_segment(insts[inst], par, N, x0, y0, z0, z1, smr);
  });
}

// ------------------------------------------------------------------------------------------
// fused_div / fused_correct: one tile column per thread; each staged plane is read once, its
// in-plane partial sums carried in z (as in fused_rhs phase 2), so the ring only has to cover
// the copies in flight: DR slots, the plane read and DR - 1 planes in flight. Rows are staged in
// 16-byte chunks starting a whole chunk left of the tile, so every chunk, wrapped or not, is one
// aligned 16-byte global segment (N is a multiple of 32).
constexpr int NTC = TX * TY;            // 512 threads
constexpr int SH = TY + 2;              // staged rows y0 - 1 .. y0 + TY
constexpr int CW = TX + 4;              // fused_correct row, float2 x0 - 2 .. x0 + TX + 1
constexpr int CPL = CW * SH;            // float2 per staged plane
constexpr int DR = 4;                   // ring slots of fused_correct
// fused_div: TX x TYD tiles and a 3-slot ring (2 planes in flight), three CTAs per SM; each slot
// holds the pairs (u*_b, P*_b) (rows x0 - 2 .. x0 + TX + 1, 16-byte chunks of 2 sites) and their
// bf16 compensations (rows x0 - 4 .. x0 + TX + 3, chunks of 4 sites)
constexpr int TYD = 16, SHD = TYD + 2, DRD = 3;
constexpr int SWP = TX + 4, SPLP = SWP * SHD;  // float2 per row, per plane
constexpr int SWL = TX + 8, SPLL = SWL * SHD;  // bf16x2 per row, per plane
constexpr size_t DIV_SLOT = 3 * SPLP * sizeof(float2) + 3 * SPLL * sizeof(__nv_bfloat162);
constexpr size_t DIV_SMEM = DRD * DIV_SLOT;
static_assert((3 * SPLP * sizeof(float2)) % 16 == 0 && DIV_SLOT % 16 == 0, "16-byte aligned staging");
static_assert(3 * DIV_SMEM <= 227 * 1024, "fused_div: three CTAs per SM");
// p_v, p_p on B; the (u*, P*) pairs and their bf16x2 compensations on C
constexpr size_t COR_SLOT = CPL * sizeof(float2) + 3 * CN * sizeof(float2) + 3 * CN * sizeof(__nv_bfloat162);
static_assert(COR_SLOT % 16 == 0 && (CPL * sizeof(float2)) % 16 == 0, "16-byte aligned ring slots");
constexpr size_t COR_SMEM = DR * COR_SLOT;
static_assert(2 * COR_SMEM <= 227 * 1024, "fused_correct: two CTAs per SM");

// wait until at most DR - 2 copy groups are pending: the group of the plane read now is complete
__device__ __forceinline__ void cp_async_wait_ring() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(DR - 2) : "memory");
}

// fused_div: 4-site strips of a 32 x 16 tile (a 6 x 3 window of each staged field serves the
// four sites), u* and P* as a packed pair.
constexpr int USD = 4;                   // sites per strip
constexpr int NTV = TX * TYD / USD;      // 128 threads
__device__ __forceinline__ void cp_async_wait_div() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(DRD - 2) : "memory");
}

// The grid of the exact part of the divergence: S = 1.5 * 2^(E + 7) with 2^E >= 2 max |v| (float
// bits of max |v|, 0: none). (v + S) - S rounds v to a multiple of g = 2^(E - 16), exactly, and the
// divergence's separable sums of such values (at most 216 x 2^16 g) stay exact in FP32.
__device__ __forceinline__ float split_grid(int mbits) {
  int e = mbits > 0 ? ((mbits >> 23) & 0xff) - 127 + 2 : -100;
  e = e < -120 ? -120 : (e > 110 ? 110 : e);
  return __int_as_float(((127 + e + 7) << 23) | 0x400000);
}

__device__ __forceinline__ void div_segment(const InstDev<float>& I, int par, int N, int x0, int y0, int z0, int z1,
                                            unsigned char* sm) {
  const size_t NN = (size_t)N * N;
  float2* const oW = I.W;
  const int stale_q2 = I.stale;
  const float kd = I.ph.c2h * (1.f / 36.f) * I.ph.inv_dt;  // d/36 of the 27-point D, and 1/dt
  const float2 S = f2(split_grid(I.smax[0]), split_grid(I.smax[1]));
  const int tid = threadIdx.x;
  const int niter = (z1 - z0) + 2;
  auto slot_p = [&](int i) { return reinterpret_cast<float2*>(sm + (i % DRD) * DIV_SLOT); };
  auto slot_l = [&](int i) {
    return reinterpret_cast<__nv_bfloat162*>(sm + (i % DRD) * DIV_SLOT + 3 * SPLP * sizeof(float2));
  };
  // issue(i): plane z0 - 1 + i into slot i % DRD (an empty group past the last plane, so that
  // every iteration commits one). Chunks outside the domain come from the previous step's u*, P*
  // when the stale-halo quirk is on (the chunk grids are aligned with 0 and N).
  // This thread's chunk items t = tid + k NTV (pair chunks first, then compensation chunks), the
  // same in every plane: the wrapped offset within a plane and the staged index, with flags for
  // a compensation chunk and for a chunk outside [0, N)^2 in (x, y). Computed once per segment.
  constexpr int CP2 = SWP / 2, CL4 = SWL / 4;  // chunks per row
  constexpr int NCH = SHD * (CP2 + CL4), KD = (NCH + NTV - 1) / NTV;
  constexpr int F_LO = 1 << 30, F_OUT = 1 << 29, F_IDX = (1 << 29) - 1;
  int goff[KD], sitem[KD];
#pragma unroll
  for (int k = 0; k < KD; ++k) {
    const int t = tid + k * NTV;
    const bool lo = t >= SHD * CP2;
    const int tt = lo ? t - SHD * CP2 : t, cr = lo ? CL4 : CP2;
    const int ry = tt / cr, rc = tt - ry * cr;
    const int gx = lo ? x0 - 4 + 4 * rc : x0 - 2 + 2 * rc, gy = y0 - 1 + ry;
    goff[k] = wrapN(gy, N) * N + wrapN(gx, N);
    sitem[k] = t >= NCH ? -1
                        : ((lo ? ry * SWL + 4 * rc : ry * SWP + 2 * rc) | (lo ? F_LO : 0) |
                           ((gx < 0 || gx >= N || gy < 0 || gy >= N) ? F_OUT : 0));
  }
  auto issue = [&](int i) {
    if (i >= niter) { cp_async_commit(); return; }
    const int zu = z0 - 1 + i;
    const bool zw = zu < 0 || zu >= N;
    const size_t zo = (size_t)wrapN(zu, N) * NN;
    float2* dp = slot_p(i);
    __nv_bfloat162* dl = slot_l(i);
#pragma unroll
    for (int k = 0; k < KD; ++k) {
      const int s = sitem[k];
      if (s < 0) continue;
      const int q = (stale_q2 && (zw || (s & F_OUT))) ? par : par ^ 1;
      const size_t g = zo + goff[k];
      const int d = s & F_IDX;
      if (s & F_LO) {
#pragma unroll
        for (int f = 0; f < 3; ++f) cp_async16(dl + f * SPLL + d, I.starlo[q][f] + g);
      } else {
#pragma unroll
        for (int f = 0; f < 3; ++f) cp_async16(dp + f * SPLP + d, I.star[q][f] + g);
      }
    }
    cp_async_commit();
  };
  const int qx = tid % TX, qy0 = (tid / TX) * USD;
  const size_t gc0 = (size_t)(y0 + qy0) * N + (x0 + qx);
  const int wbp = qy0 * SWP + (qx + 1);  // staged pair index of window row 0, column x - 1
  const int wbl = qy0 * SWL + (qx + 3);  // the same in the compensation rows
  // the divergence D_x v_x + D_y v_y + D_z v_z of v = (u*, P*) (getStream mode 0, :664-670), each
  // D = d/36 delta s s: a plane adds Q = delta_x s_y v_x + s_x delta_y v_y with weight s_z =
  // (1, 4, 1) and Z = s_x s_y v_z with weight delta_z = (-1, 0, 1) over planes c-1, c, c+1.
  // It is taken in two parts, exactly: v = q + s with q the FP32 value rounded to the grid of
  // split_grid, whose sums are exact, and s the rest (the FP32 value's remainder plus the bf16
  // compensation), small enough that its sums' rounding is negligible. u* is nearly solenoidal,
  // so its divergence is a small difference of large values; taken plainly in FP32 its rounding,
  // amplified by 1/dt, would dominate the pressure.
  float2 rD1[2][USD], rD2[2][USD];  // [part][site]
#pragma unroll
  for (int k = 0; k < USD; ++k) rD1[0][k] = rD2[0][k] = rD1[1][k] = rD2[1][k] = f2(0.f, 0.f);
  float amx = 0.f, amy = 0.f;  // max |Re W|, |Im W| of this thread's outputs
  const float2 four = f2(4.f, 4.f);
  auto split = [&](float2 hi, __nv_bfloat162 lo, float2& q, float2& rest) {
    q = vsub(vadd(hi, S), S);
    rest = vadd(vsub(hi, q), __bfloat1622float2(lo));
  };
#pragma unroll
  for (int k = 0; k < DRD - 1; ++k) issue(k);
  for (int i = 0; i < niter; ++i) {
    cp_async_wait_div();
    __syncthreads();
    issue(i + DRD - 1);  // into the slot read at iteration i - 1
    const float2* sp = slot_p(i) + wbp;
    const __nv_bfloat162* sl = slot_l(i) + wbl;
    // the three columns x - 1, x, x + 1 of component f in window row r, split (one 8-byte load
    // per column of the pairs and one 4-byte load of the compensations: the same shared-memory
    // wavefronts as wider aligned loads, without lane-dependent selects)
    auto row3 = [&](int f, int r, float2* q, float2* rest) {
      const float2* a = sp + f * SPLP + r * SWP;
      const __nv_bfloat162* b = sl + f * SPLL + r * SWL;
#pragma unroll
      for (int c = 0; c < 3; ++c) split(a[c], b[c], q[c], rest[c]);
    };
    // per row of the window and part: the x-part delta_x v_x, and s_x of v_y and of v_z
    float2 xd[2][USD + 2], ys[2][USD + 2], zs[2][USD + 2];
#pragma unroll
    for (int r = 0; r < USD + 2; ++r) {
      float2 q0, s0, q2, s2;
      split(sp[r * SWP], sl[r * SWL], q0, s0);
      split(sp[r * SWP + 2], sl[r * SWL + 2], q2, s2);
      xd[0][r] = vsub(q2, q0);
      xd[1][r] = vsub(s2, s0);
      float2 qc[3], rc[3];
      row3(1, r, qc, rc);
      ys[0][r] = vfma(four, qc[1], vadd(qc[0], qc[2]));
      ys[1][r] = vfma(four, rc[1], vadd(rc[0], rc[2]));
      row3(2, r, qc, rc);
      zs[0][r] = vfma(four, qc[1], vadd(qc[0], qc[2]));
      zs[1][r] = vfma(four, rc[1], vadd(rc[0], rc[2]));
    }
#pragma unroll
    for (int k = 0; k < USD; ++k) {
      float2 dvp[2];
#pragma unroll
      for (int pt = 0; pt < 2; ++pt) {
        const float2 xr = vfma(four, xd[pt][k + 1], vadd(xd[pt][k], xd[pt][k + 2]));  // delta_x s_y v_x
        const float2 yr = vsub(ys[pt][k + 2], ys[pt][k]);                               // s_x delta_y v_y
        const float2 zr = vfma(four, zs[pt][k + 1], vadd(zs[pt][k], zs[pt][k + 2]));    // s_x s_y v_z
        const float2 Q = vadd(xr, yr);
        dvp[pt] = vadd(vadd(rD1[pt][k], Q), zr);
        rD1[pt][k] = vfma(four, Q, rD2[pt][k]);
        rD2[pt][k] = vsub(Q, zr);
      }
      if (i >= 2) {
        const float2 wv = vmul(vsplat(kd, float2()), vadd(dvp[0], dvp[1]));
        oW[(size_t)(z0 - 2 + i) * NN + gc0 + (size_t)k * N] = wv;
        amx = fmaxf(amx, fabsf(wv.x));
        amy = fmaxf(amy, fabsf(wv.y));
      }
    }
  }
  record_wmax(I.wmax, amx, amy);
}

template <bool PERSIST>
__global__ void __launch_bounds__(NTV, 3) k_fused_div(const InstDev<float>* __restrict__ insts, int par, int nchunk, int zc,
                                                       int ninst) {
  extern __shared__ __align__(16) unsigned char smd[];
  const int N = insts[0].N;
  sweep_schedule<TX, TYD, PERSIST>(N, nchunk, zc, ninst, [&](int inst, int x0, int y0, int z0, int z1) {
    div_segment(insts[inst], par, N, x0, y0, z0, z1, smd);
  });
}

__device__ __forceinline__ void correct_segment(const InstDev<float>& I, int par, int N, int x0, int y0, int z0, int z1,
                                                unsigned char* smc) {
  const float kd = I.ph.c2h * (1.f / 36.f);
  const float dt = I.ph.dt;
  // the pressures come out of the FFT scaled by powers of two (pow2_norm): undo it, exactly
  const float du = pow2_denorm(I.wmax[0]), dp = pow2_denorm(I.wmax[1]);
  const size_t NN = (size_t)N * N;
  const int niter = (z1 - z0) + 2;
  float* const oU[3] = {I.U[0], I.U[1], I.U[2]};
  float* const oP[3] = {I.P[0], I.P[1], I.P[2]};
  const float2* __restrict__ gW = I.W;
  const int tid = threadIdx.x;
  auto slot_w = [&](int i) { return reinterpret_cast<float2*>(smc + (i % DR) * COR_SLOT); };
  auto slot_q = [&](int i) { return reinterpret_cast<float2*>(smc + (i % DR) * COR_SLOT + CPL * sizeof(float2)); };
  auto slot_l = [&](int i) {
    return reinterpret_cast<__nv_bfloat162*>(smc + (i % DR) * COR_SLOT + CPL * sizeof(float2) + 3 * CN * sizeof(float2));
  };
  // issue(i): into slot i % DR the pressures (p_v, p_p) of plane z0 - 1 + i over tile+1 and u*, P*
  // of plane z0 - 2 + i (finished at iteration i) with their compensations over the tile; an empty
  // group past the last plane
  auto issue = [&](int i) {
    if (i >= niter) { cp_async_commit(); return; }
    const int zz = wrapN(z0 - 1 + i, N);
    float2* dst = slot_w(i);
    constexpr int CR = CW / 2;  // chunks per row
    for (int t = tid; t < SH * CR; t += NTC) {
      const int ry = t / CR, rc = t - ry * CR;
      cp_async16(dst + ry * CW + 2 * rc,
                 gW + (size_t)zz * NN + (size_t)wrapN(y0 - 1 + ry, N) * N + wrapN(x0 - 2 + 2 * rc, N));
    }
    const int zq = z0 - 2 + i;
    if (zq >= z0) {
      // the pairs (u*_b, P*_b) over the tile: 16-byte chunks of 2 sites
      float2* dq = slot_q(i);
      constexpr int QR = TX / 2, QF = TY * QR;  // chunks per tile row, per pair field
      for (int t = tid; t < 3 * QF; t += NTC) {
        const int f = t / QF, r = t - f * QF;
        const int ry = r / QR, rc = r - ry * QR;
        cp_async16(dq + f * CN + ry * TX + 2 * rc, I.star[par ^ 1][f] + (size_t)zq * NN + (size_t)(y0 + ry) * N + x0 + 2 * rc);
      }
      // their compensations: 16-byte chunks of 4 sites
      __nv_bfloat162* dl = slot_l(i);
      constexpr int LR = TX / 4, LF = TY * LR;  // chunks per tile row, per field
      for (int t = tid; t < 3 * LF; t += NTC) {
        const int f = t / LF, r = t - f * LF;
        const int ry = r / LR, rc = r - ry * LR;
        cp_async16(dl + f * CN + ry * TX + 4 * rc,
                   I.starlo[par ^ 1][f] + (size_t)zq * NN + (size_t)(y0 + ry) * N + x0 + 4 * rc);
      }
    }
    cp_async_commit();
  };
  const int qx = tid % TX, qy = tid / TX;
  const size_t gc = (size_t)(y0 + qy) * N + (x0 + qx);
  // gradients D_a of p_v and p_p, D = d/36 delta s s: a plane adds X = delta_x s_y p and
  // Y = s_x delta_y p with weight s_z = (1, 4, 1), Z = s_x s_y p with weight delta_z = (-1, 0, 1)
  float2 rX1 = make_float2(0.f, 0.f), rX2 = rX1, rY1 = rX1, rY2 = rX1, rZ1 = rX1, rZ2 = rX1;
#pragma unroll
  for (int k = 0; k < DR - 1; ++k) issue(k);
  for (int i = 0; i < niter; ++i) {
    cp_async_wait_ring();
    __syncthreads();
    issue(i + DR - 1);  // into the slot read at iteration i - 1
    const float2* s = slot_w(i) + (qy + 1) * CW + (qx + 2);
    float2 v[3][3];
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
      for (int c = 0; c < 3; ++c) v[r][c] = s[(r - 1) * CW + (c - 1)];
    float2 gx, gy, gz;
#define TTSH_PLANE(C)                                                                                          \
    {                                                                                                          \
      const float X = fmaf(4.f, v[1][2].C - v[1][0].C, (v[0][2].C - v[0][0].C) + (v[2][2].C - v[2][0].C));     \
      const float Y = fmaf(4.f, v[2][1].C - v[0][1].C, (v[2][0].C - v[0][0].C) + (v[2][2].C - v[0][2].C));     \
      const float t0 = fmaf(4.f, v[1][0].C, v[0][0].C + v[2][0].C);                                            \
      const float t1 = fmaf(4.f, v[1][1].C, v[0][1].C + v[2][1].C);                                            \
      const float t2 = fmaf(4.f, v[1][2].C, v[0][2].C + v[2][2].C);                                            \
      const float Z = fmaf(4.f, t1, t0 + t2);                                                                  \
      gx.C = rX1.C + X; rX1.C = fmaf(4.f, X, rX2.C); rX2.C = X;                                                \
      gy.C = rY1.C + Y; rY1.C = fmaf(4.f, Y, rY2.C); rY2.C = Y;                                                \
      gz.C = rZ1.C + Z; rZ1.C = rZ2.C; rZ2.C = -Z;                                                             \
    }
    TTSH_PLANE(x)
    TTSH_PLANE(y)
#undef TTSH_PLANE
    if (i >= 2) {
      // getVNew (TTSH3D.cu:505-511): u = u* - dt D p_v, P = P* - dt D p_p
      const size_t g = (size_t)(z0 - 2 + i) * NN + gc;
      const float2* qc = slot_q(i) + qy * TX + qx;
      const __nv_bfloat162* lc = slot_l(i) + qy * TX + qx;
      const float gv[3] = {gx.x, gy.x, gz.x}, gp[3] = {gx.y, gy.y, gz.y};
      // u compensated: the FP32 value and, in bf16, what its rounding dropped plus u*'s
      // compensation. P: the FP32 value nearest the exact P* - dt D p_p (its compensation is not
      // kept: carried from step to step it would also integrate the FP32 rounding of P's update
      // where that update is a small difference of its large terms, |P| near its equilibrium,
      // increments that an FP32 state drops)
#pragma unroll
      for (int b = 0; b < 3; ++b) {
        const float2 st = qc[b * CN];
        const __nv_bfloat162 sl = lc[b * CN];
        put_comp(oU[b], I.lo[b], g, st.x, -(dt * (kd * (gv[b] * du))), __low2bfloat16(sl));
        float e;
        const float v = two_sum(st.y, -(dt * (kd * (gp[b] * dp))), e);
        oP[b][g] = v + (e + __bfloat162float(__high2bfloat16(sl)));
      }
    }
  }
}

template <bool PERSIST>
__global__ void __launch_bounds__(NTC, 2) k_fused_correct(const InstDev<float>* __restrict__ insts, int par, int nchunk,
                                                          int zc, int ninst) {
  extern __shared__ __align__(16) unsigned char smc[];
  const int N = insts[0].N;
  // the next step's maxima of u*, P* start from zero (fused_rhs records them; fused_div, which
  // reads them, ran before this kernel)
  if (blockIdx.x == 0 && blockIdx.y == 0 && blockIdx.z == 0)
    for (int i = threadIdx.x; i < 2 * ninst; i += blockDim.x) insts[i >> 1].smax[i & 1] = 0;
  sweep_schedule<TX, TY, PERSIST>(N, nchunk, zc, ninst, [&](int inst, int x0, int y0, int z0, int z1) {
    correct_segment(insts[inst], par, N, x0, y0, z0, z1, smc);
  });
}

inline void check(cudaError_t e, const char* what) {
  if (e != cudaSuccess) throw std::runtime_error(std::string(what) + ": " + cudaGetErrorString(e));
}

dim3 grid_for(const Group<float>& g, int zc, int& nchunk) {
  if (zc < 1) throw std::runtime_error("fused: z-planes per block must be >= 1");
  nchunk = (g.N + zc - 1) / zc;
  if ((long)nchunk * g.n > 65535) throw std::runtime_error("fused: too many droplets in one group");
  return dim3(g.N / TX, g.N / TY, nchunk * g.n);
}

}  // namespace

bool fused_supported(int N) { return N >= 32 && N % TX == 0 && N % TY == 0 && N % TYD == 0; }

void fused_prepare() {
  const std::pair<const void*, size_t> k[] = {
      {(const void*)k_fused_rhs<false>, RHS_SMEM},     {(const void*)k_fused_rhs<true>, RHS_SMEM},
      {(const void*)k_fused_div<false>, DIV_SMEM},     {(const void*)k_fused_div<true>, DIV_SMEM},
      {(const void*)k_fused_correct<false>, COR_SMEM}, {(const void*)k_fused_correct<true>, COR_SMEM}};
  for (const auto& f : k)
    check(cudaFuncSetAttribute(f.first, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)f.second),
          "fused kernels' smem attribute");
}

// The persistent grid of a fused kernel (zc == 0): the CTAs that fit on the device at once, at
// most one per plane of a tile column.
static int persistent_grid(const void* kernel, int threads, size_t smem, long long planes, int* cache) {
  if (!*cache) {
    int dev = 0, sms = 0, per = 0;
    check(cudaGetDevice(&dev), "fused: device");
    check(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev), "fused: SM count");
    check(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kernel, threads, smem), "fused: occupancy");
    if (per < 1) throw std::runtime_error("fused: kernel does not fit on an SM");
    *cache = sms * per;
  }
  return (int)std::min<long long>(*cache, planes);
}

template <class K>
static void launch_sweep(K chunked, K persistent, const Group<float>& g, int par, int zc, int th, int threads, size_t smem,
                         int* cache, cudaStream_t st, const char* what) {
  if (zc == 0) {
    const long long planes = (long long)g.n * (g.N / TX) * (g.N / th) * g.N;
    const int grid = persistent_grid((const void*)persistent, threads, smem, planes, cache);
    persistent<<<grid, threads, smem, st>>>(g.d_inst, par, 1, 0, g.n);
  } else {
    int nchunk;
    dim3 grid = grid_for(g, zc, nchunk);
    grid.y = g.N / th;
    chunked<<<grid, threads, smem, st>>>(g.d_inst, par, nchunk, zc, g.n);
  }
  check(cudaGetLastError(), what);
}

void launch_fused_rhs(const Group<float>& g, int par, cudaStream_t st) {
  static int cache = 0;
  launch_sweep(k_fused_rhs<false>, k_fused_rhs<true>, g, par, g.zc[0], TYR, NT, RHS_SMEM, &cache, st, "fused_rhs launch");
}

void launch_fused_div(const Group<float>& g, int par, cudaStream_t st) {
  static int cache = 0;
  launch_sweep(k_fused_div<false>, k_fused_div<true>, g, par, g.zc[1], TYD, NTV, DIV_SMEM, &cache, st, "fused_div launch");
}

void launch_fused_correct(const Group<float>& g, int par, cudaStream_t st) {
  static int cache = 0;
  launch_sweep(k_fused_correct<false>, k_fused_correct<true>, g, par, g.zc[2], TY, NTC, COR_SMEM, &cache, st, "fused_correct launch");
}

}  // namespace ttsh
