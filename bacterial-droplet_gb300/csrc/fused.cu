// fused.cu — the fused FP32 form of the TTSH3D step.
//
// Three kernels replace stage1 + stage2 + div + correct of the plain form (plain.cu):
//
//   fused_rhs     phi, P, u -> u*, P*, phi'   (getTempVari_1/2 + getDtF + getVStar + the phi
//                 update of getVNew, TTSH3D.cu:537-632, :471-491, :515), all intermediates
//                 (mu_0, mu_b, the stress S_ab, D_a P_b) kept in shared memory.
//   fused_div     u*, P* -> W = div(u*)/dt + i div(P*)/dt   (getStream mode 0, :664-670, with
//                 the reference's stale halo for neighbours across the periodic boundary)
//   fused_correct u*, P*, W -> u, P   (getVNew, :505-511)
//
// All three march along z through a tile of TX x TY columns (a "2.5D" sweep): each z-plane of
// every field the stencils need is staged once in a shared-memory ring of planes, and each
// thread evaluates the 27-point derivatives / 15-point Laplacians of a 1 x R strip of sites
// from registers (the strip's 3 x (R+2) x 3 neighbourhood), so warps read shared memory with
// unit stride. The nested stencils of the RHS (sigma and mu need D P and L P; the velocity
// update needs D sigma and L mu) are staged: stage 1 forms the products of plane z+1 while
// the thread of each tile column finishes plane z. It splits those outer stencils into
// in-plane partial sums and carries the z-combination in registers from plane to plane,
// so every product plane is read once.
//
// The stencil arithmetic is the reference's (st_dx/st_dy/st_dz/st_lap of common.cuh) in FP32;
// the stress enters as one field per component, S_ab = cA phi D_a P_b - zeta phi P_a P_b, whose
// divergence is the reference's cA * div(sigma) plus the build-defined active stress.
#include <cstdio>
#include <stdexcept>

#include "common.cuh"
#include "kernels.h"

namespace ttsh {

namespace {

constexpr int TX = 32, TY = 16;   // output tile (columns)
constexpr int ZC = 64;            // z-planes per block (chunk)
constexpr int RB = 2;             // strip length (sites per thread) of fused_rhs stage 1
constexpr int NT = 512;           // threads of fused_rhs: one tile column each in stage 2
constexpr int US = 4;             // strip length of the velocity terms (phase 1)

// fused_rhs regions: A = tile + 2 (phi, P), B = tile + 1 (u, stage-1 products), C = tile.
constexpr int AW = TX + 4, AH = TY + 4, AN = AW * AH;
constexpr int BW = TX + 2, BH = TY + 2, BN = BW * BH;
constexpr int CN = TX * TY;
// stage-1 products of one plane on B, and the pointwise parts of the update ("partials") on C
constexpr int QS = 0, QMU = 9, QMU0 = 12, NQ = 13;
constexpr int PU = 0, PP = 3, PPHI = 6;
// Shared memory (floats): A ring RA planes x 4 fields; u ring RU x 3; one plane of the 13
// products; partials ring 2 planes x 7. The A and u rings hold one plane more than the stencils
// read: the next plane is copied into it (cp.async) while the current ones compute.
constexpr int RA = 4, RU = 4;
constexpr int SA_OFF = 0;
constexpr int SU_OFF = SA_OFF + RA * 4 * AN;
constexpr int SB_OFF = SU_OFF + RU * 3 * BN;
constexpr int SQ_OFF = SB_OFF + NQ * BN;
constexpr int RHS_SMEM_FLOATS = SQ_OFF + 2 * 7 * CN;
constexpr size_t RHS_SMEM = RHS_SMEM_FLOATS * sizeof(float);
// phase-1 thread roles of fused_rhs: stage-1 strips of the B region, then the velocity strips
constexpr int NS1 = (BW * BH) / RB;                   // 306 stage-1 strips
constexpr int NU0 = ((NS1 + 31) / 32) * 32;           // first velocity thread (warp aligned)
constexpr int NUS = TX * (TY / US);                   // 128 velocity strips
static_assert((BH % RB) == 0 && (TY % US) == 0, "strip lengths divide the regions");
static_assert(NU0 + NUS <= NT, "phase-1 roles fit the block");

__device__ __forceinline__ int wrapN(int a, int N) { return a < 0 ? a + N : (a >= N ? a - N : a); }

// Asynchronous global -> shared copies (cp.async): the data lands while the CTA computes.
__device__ __forceinline__ void cp_async4(void* smem, const void* gmem) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async8(void* smem, const void* gmem) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;\n" ::: "memory"); }

// A 3 (planes) x (R+2) (rows) x 3 (columns) neighbourhood held in registers, for a strip of R
// sites stacked in y. F(dx,dy,dz) of site k reads v[1+dz][1+k+dy][1+dx].
template <int R>
struct Hood {
  float v[3][R + 2][3];
  __device__ __forceinline__ void load(const float* p0, const float* p1, const float* p2, int W, int x, int y0) {
    const float* pl[3] = {p0, p1, p2};
#pragma unroll
    for (int z = 0; z < 3; ++z)
#pragma unroll
      for (int r = 0; r < R + 2; ++r)
#pragma unroll
        for (int c = 0; c < 3; ++c) v[z][r][c] = pl[z][(y0 - 1 + r) * W + (x - 1 + c)];
  }
};
template <int R>
struct HoodAcc {
  const Hood<R>* h;
  int k;
  __device__ __forceinline__ float operator()(int dx, int dy, int dz) const { return h->v[1 + dz][1 + k + dy][1 + dx]; }
};

// Separable evaluation on a Hood (FP32 form). With s = [1, 4, 1] and delta = [-1, 0, 1]:
//   D_x = c2h/36 * delta_x s_y s_z,  D_y = c2h/36 * s_x delta_y s_z,  D_z = c2h/36 * s_x s_y delta_z,
//   L = cl12 * (8 corners) + cl23 * (6 faces) - cl143 * centre  (corners = c_x c_y c_z, c = [1, 0, 1]),
// the reference's 27-point and 15-point weights (TTSH3D.cu:3280-3343) regrouped so that the
// z-combinations of each (row, column) are shared by the R sites of the strip.
struct SepK {
  float d;  // c2h / 36
  float l12, l23, l143;
};
template <int R, bool DX, bool DY, bool DZ, bool LAP>
__device__ __forceinline__ void sep_eval(const Hood<R>& h, const SepK& k, float* dx, float* dy, float* dz, float* lap) {
  float cz[R + 2][3], sz[R + 2][3], dzr[R + 2][3];
#pragma unroll
  for (int r = 0; r < R + 2; ++r)
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      cz[r][c] = h.v[0][r][c] + h.v[2][r][c];
      sz[r][c] = fmaf(4.f, h.v[1][r][c], cz[r][c]);
      dzr[r][c] = h.v[2][r][c] - h.v[0][r][c];
    }
#pragma unroll
  for (int i = 0; i < R; ++i) {
    if (DX) {
      const float a = fmaf(4.f, sz[i + 1][2], sz[i][2] + sz[i + 2][2]);
      const float b = fmaf(4.f, sz[i + 1][0], sz[i][0] + sz[i + 2][0]);
      dx[i] = k.d * (a - b);
    }
    if (DY) {
      const float e0 = sz[i + 2][0] - sz[i][0], e1 = sz[i + 2][1] - sz[i][1], e2 = sz[i + 2][2] - sz[i][2];
      dy[i] = k.d * fmaf(4.f, e1, e0 + e2);
    }
    if (DZ) {
      const float f0 = fmaf(4.f, dzr[i + 1][0], dzr[i][0] + dzr[i + 2][0]);
      const float f1 = fmaf(4.f, dzr[i + 1][1], dzr[i][1] + dzr[i + 2][1]);
      const float f2 = fmaf(4.f, dzr[i + 1][2], dzr[i][2] + dzr[i + 2][2]);
      dz[i] = k.d * fmaf(4.f, f1, f0 + f2);
    }
    if (LAP) {
      const float corners = (cz[i][0] + cz[i][2]) + (cz[i + 2][0] + cz[i + 2][2]);
      const float faces = (cz[i + 1][1] + h.v[1][i + 1][0]) + (h.v[1][i + 1][2] + h.v[1][i][1]) + h.v[1][i + 2][1];
      lap[i] = fmaf(k.l12, corners, fmaf(k.l23, faces, -k.l143 * h.v[1][i + 1][1]));
    }
  }
}

// Interleaved-complex variant (one component of a float2 plane).
template <int R>
struct Hood2 {
  float2 v[3][R + 2][3];
  __device__ __forceinline__ void load(const float2* p0, const float2* p1, const float2* p2, int W, int x, int y0) {
    const float2* pl[3] = {p0, p1, p2};
#pragma unroll
    for (int z = 0; z < 3; ++z)
#pragma unroll
      for (int r = 0; r < R + 2; ++r)
#pragma unroll
        for (int c = 0; c < 3; ++c) v[z][r][c] = pl[z][(y0 - 1 + r) * W + (x - 1 + c)];
  }
};
template <int R, int COMP>
struct Hood2Acc {
  const Hood2<R>* h;
  int k;
  __device__ __forceinline__ float operator()(int dx, int dy, int dz) const {
    const float2 t = h->v[1 + dz][1 + k + dy][1 + dx];
    return COMP == 0 ? t.x : t.y;
  }
};

// ------------------------------------------------------------------------------------------
__global__ void __launch_bounds__(NT, 1) k_fused_rhs(const InstDev<float>* __restrict__ insts, int par, int nchunk) {
  extern __shared__ __align__(16) float sm[];
  const int N = insts[0].N;
  const InstDev<float>& I = insts[blockIdx.z / nchunk];
  const Phys<float> p = I.ph;  // by value: read once, kept in registers
  const SepK sk{p.c2h * (1.f / 36.f), p.cl12, p.cl23, p.cl143};
  const int x0 = blockIdx.x * TX, y0 = blockIdx.y * TY;
  const int z0 = (blockIdx.z % nchunk) * ZC;
  const int z1 = min(z0 + ZC, N);
  const size_t NN = (size_t)N * N;
  const float* __restrict__ gphi = I.phi[par];
  const float* __restrict__ gP[3] = {I.P[0], I.P[1], I.P[2]};
  const float* __restrict__ gU[3] = {I.U[0], I.U[1], I.U[2]};
  float* const oUs[3] = {I.Us[par ^ 1][0], I.Us[par ^ 1][1], I.Us[par ^ 1][2]};
  float* const oPs[3] = {I.Ps[par ^ 1][0], I.Ps[par ^ 1][1], I.Ps[par ^ 1][2]};
  float* const ophi = I.phi[par ^ 1];
  float* const phic = I.phic;
  float* sA = sm + SA_OFF;  // [RA][4][AN]: phi, Px, Py, Pz
  float* sU = sm + SU_OFF;  // [RU][3][BN]
  float* sB = sm + SB_OFF;  // [NQ][BN]: products of plane b
  float* sQ = sm + SQ_OFF;  // [2][7][CN]
  const int tid = threadIdx.x;
  const int niter = (z1 - z0) + 4;

  // issue(i): A plane a = z0 - 2 + i (phi, P over tile+2) into A slot i % RA, and u plane a - 1
  // (tile+1) into u slot i % RU. Iteration i runs stage 1 at plane b = a - 1 and finishes plane
  // c = a - 2; issue(i + 1) runs during iteration i.
  auto issue = [&](int i) {
    const int za = ((z0 - 2 + i) % N + N) % N;
    float* dst = sA + (i % RA) * 4 * AN;
    for (int t = tid; t < AN; t += NT) {
      const int ay = t / AW, ax = t - ay * AW;
      const size_t g = (size_t)za * NN + (size_t)wrapN(y0 - 2 + ay, N) * N + wrapN(x0 - 2 + ax, N);
      cp_async4(dst + t, gphi + g);
      cp_async4(dst + AN + t, gP[0] + g);
      cp_async4(dst + 2 * AN + t, gP[1] + g);
      cp_async4(dst + 3 * AN + t, gP[2] + g);
    }
    const int zu = ((z0 - 3 + i) % N + N) % N;
    float* du = sU + (i % RU) * 3 * BN;
    for (int t = tid; t < BN; t += NT) {
      const int by = t / BW, bx = t - by * BW;
      const size_t g = (size_t)zu * NN + (size_t)wrapN(y0 - 1 + by, N) * N + wrapN(x0 - 1 + bx, N);
      cp_async4(du + t, gU[0] + g);
      cp_async4(du + BN + t, gU[1] + g);
      cp_async4(du + 2 * BN + t, gU[2] + g);
    }
    cp_async_commit();
  };
  // the tile column of this thread in phase 2
  const int qx = tid % TX, qy = tid / TX;
  const size_t gc = (size_t)(y0 + qy) * N + (x0 + qx);
  const int qo = (qy + 1) * BW + (qx + 1);  // its B-region index
  // z-combinations carried from plane to plane (phase 2): for the Laplacians of mu_b, mu_0,
  // rL1 = the partial sum of the plane just finished + 1, rL2 = that of the plane after it;
  // likewise rD1 / rD2 for the stress divergence of column b
  float rL1[4] = {0.f, 0.f, 0.f, 0.f}, rL2[4] = {0.f, 0.f, 0.f, 0.f};
  float rD1[3] = {0.f, 0.f, 0.f}, rD2[3] = {0.f, 0.f, 0.f};
  issue(0);
  for (int i = 0; i < niter; ++i) {
    cp_async_wait_all();
    __syncthreads();
    if (i + 1 < niter) issue(i + 1);
    // the phi compensation of this iteration's output site, loaded before phase 1 so that the
    // phase-1 work covers the load
    const float cprev = i >= 4 ? phic[(size_t)(z0 - 4 + i) * NN + gc] : 0.f;
    // ---- phase 1a, stage 1 at plane b = z0 - 3 + i over B (tile+1): the products mu_0, mu_b,
    //      S_ab that phase 2 differentiates, and on the tile the pointwise parts of the update
    if (i >= 2 && tid < NS1) {
      const float* a0 = sA + ((i + RA - 2) % RA) * 4 * AN;  // plane b-1
      const float* a1 = sA + ((i + RA - 1) % RA) * 4 * AN;  // plane b
      const float* a2 = sA + (i % RA) * 4 * AN;             // plane b+1
      const float* ub = sU + (i % RU) * 3 * BN;             // u at plane b
      float* bq = sB;
      float* pq = sQ + (i & 1) * 7 * CN;
      // strips of the B region: warps take 32 consecutive columns of one strip row (unit-stride
      // shared-memory access); the last BW - 32 columns of every row come after them
      constexpr int NSR = BH / RB, NMAIN = 32 * NSR;
      const int s = tid;
      int bx, by0;
      if (s < NMAIN) { bx = s & 31; by0 = (s >> 5) * RB; }
      else { const int e = s - NMAIN; bx = 32 + e % (BW - 32); by0 = (e / (BW - 32)) * RB; }
      const int ax = bx + 1, ay0 = by0 + 1;  // A coordinates
      float phc[RB], lphi[RB], dphi[3][RB];
      {
        Hood<RB> h;
        h.load(a0, a1, a2, AW, ax, ay0);
#pragma unroll
        for (int k = 0; k < RB; ++k) phc[k] = h.v[1][1 + k][1];
        sep_eval<RB, true, true, true, true>(h, sk, dphi[0], dphi[1], dphi[2], lphi);
      }
      float Pc[3][RB], DP[3][3][RB];  // DP[a][b] = D_a P_b
#pragma unroll
      for (int b = 0; b < 3; ++b) {
        Hood<RB> h;
        h.load(a0 + (1 + b) * AN, a1 + (1 + b) * AN, a2 + (1 + b) * AN, AW, ax, ay0);
        float lp[RB];
        sep_eval<RB, true, true, true, true>(h, sk, DP[0][b], DP[1][b], DP[2][b], lp);
#pragma unroll
        for (int k = 0; k < RB; ++k) {
          Pc[b][k] = h.v[1][1 + k][1];
          bq[(QMU + b) * BN + (by0 + k) * BW + bx] = fmaf(p.La2, lp[k], phc[k] * Pc[b][k]);  // mu_b (:571-573)
        }
      }
#pragma unroll
      for (int k = 0; k < RB; ++k) {
        const float ph = phc[k];
        const int o = (by0 + k) * BW + bx;
        const float mu0 = p.aPhi2 * (ph - 3 * ph * ph + 2 * ph * ph * ph) - p.kPhi * lphi[k];  // mu_0 (:567)
        bq[QMU0 * BN + o] = mu0;
#pragma unroll
        for (int a = 0; a < 3; ++a)
#pragma unroll
          for (int b = 0; b < 3; ++b) {
            float sv = p.cA * (ph * DP[a][b][k]);  // cA * sigma_ab (:587-595)
            if (p.zeta != 0.f) sv -= p.zeta * (ph * Pc[a][k] * Pc[b][k]);
            bq[(QS + a * 3 + b) * BN + o] = sv;
          }
        const int cx = bx - 1, cy = by0 + k - 1;
        if (cx >= 0 && cx < TX && cy >= 0 && cy < TY) {
          // pointwise parts of getDtF (:617-631) at this site of plane b
          const int c = cy * TX + cx;
          const float vx = ub[o], vy = ub[BN + o], vz = ub[2 * BN + o];
          const float px = Pc[0][k], py = Pc[1][k], pz = Pc[2][k];
          const float P2 = px * px + py * py + pz * pz;
          const float dPhi2 = dphi[0][k] * dphi[0][k] + dphi[1][k] * dphi[1][k] + dphi[2][k] * dphi[2][k];
#pragma unroll
          for (int b = 0; b < 3; ++b) {
            pq[(PU + b) * CN + c] = mu0 * dphi[b][k];  // mu_0 D_b phi
            const float pb = Pc[b][k];
            float cub;
            if (b == 0) cub = px * px * px + px * py * py + px * pz * pz;
            else if (b == 1) cub = px * py * px + py * py * py + py * pz * pz;
            else cub = px * pz * px + py * pz * py + pz * pz * pz;
            const float Ab = dphi[0][k] * dphi[b][k] * px + dphi[1][k] * dphi[b][k] * py + dphi[2][k] * dphi[b][k] * pz;
            pq[(PP + b) * CN + c] = -vx * DP[0][b][k] - vy * DP[1][b][k] - vz * DP[2][b][k] - p.alpha * ph * pb -
                                    p.beta * P2 * pb - p.lambda0 * (px * DP[0][b][k] + py * DP[1][b][k] + pz * DP[2][b][k]) -
                                    p.A * (dPhi2 * cub + sqrtf(P2) * Ab);
          }
          pq[PPHI * CN + c] = -vx * dphi[0][k] - vy * dphi[1][k] - vz * dphi[2][k];
        }
      }
    }
    // ---- phase 1b, on the threads stage 1 leaves free: the velocity terms of plane c = b - 1,
    //      -u.D u_b + mu L u_b (:617-621), added to that plane's partials (written by stage 1 at
    //      iteration i - 1), for a strip of US sites of one tile column
    if (i >= 4 && tid >= NU0 && tid < NU0 + NUS) {
      const int s = tid - NU0;
      const int vx = s & 31, vy0 = (s >> 5) * US;  // tile coordinates of the strip
      const float* u0 = sU + ((i + RU - 2) % RU) * 3 * BN;  // plane c-1
      const float* u1 = sU + ((i + RU - 1) % RU) * 3 * BN;  // plane c
      const float* u2 = sU + (i % RU) * 3 * BN;             // plane c+1
      float* pq = sQ + ((i + 1) & 1) * 7 * CN;
      float uc[3][US];
#pragma unroll
      for (int b = 0; b < 3; ++b)
#pragma unroll
        for (int k = 0; k < US; ++k) uc[b][k] = u1[b * BN + (vy0 + 1 + k) * BW + vx + 1];
#pragma unroll
      for (int b = 0; b < 3; ++b) {
        float dx[US], dy[US], dz[US], lu[US];
        {
          Hood<US> h;
          h.load(u0 + b * BN, u1 + b * BN, u2 + b * BN, BW, vx + 1, vy0 + 1);
          sep_eval<US, true, true, true, true>(h, sk, dx, dy, dz, lu);
        }
#pragma unroll
        for (int k = 0; k < US; ++k)
          pq[(PU + b) * CN + (vy0 + k) * TX + vx] +=
              -uc[0][k] * dx[k] - uc[1][k] * dy[k] - uc[2][k] * dz[k] + p.mu * lu[k];
      }
    }
    __syncthreads();
    // ---- phase 2, one tile column per thread: the in-plane partial sums of the outer stencils
    //      over the products of plane b, carried in z; plane c = b - 1 is then complete
    if (i >= 2) {
      const float* bq = sB + qo;
      // 15-point Laplacian L = l12 (8 corners) + l23 (6 faces) - l143 (centre) (:3328-3343):
      // an off-centre plane p adds G_p = l12 (its 4 diagonal sites) + l23 (its centre site),
      // the centre plane adds H_p = l23 (its 4 edge sites) - l143 (its centre site)
      float lmu[4];
#pragma unroll
      for (int f = 0; f < 4; ++f) {
        const float* F = bq + (QMU + f) * BN;
        const float v11 = F[0];
        const float dg = (F[-BW - 1] + F[-BW + 1]) + (F[BW - 1] + F[BW + 1]);
        const float ed = (F[-BW] + F[BW]) + (F[-1] + F[1]);
        const float G = fmaf(sk.l12, dg, sk.l23 * v11);
        const float H = fmaf(sk.l23, ed, -sk.l143 * v11);
        lmu[f] = rL1[f] + G;
        rL1[f] = rL2[f] + H;
        rL2[f] = G;
      }
      // divergence of stress column b, d/36 (delta_x s_y s_z S_xb + s_x delta_y s_z S_yb +
      // s_x s_y delta_z S_zb): the plane adds Q = delta_x s_y S_xb + s_x delta_y S_yb with weight
      // s_z = (1, 4, 1) and Z = s_x s_y S_zb with weight delta_z = (-1, 0, 1) over planes c-1, c, c+1
      float dv[3];
#pragma unroll
      for (int b = 0; b < 3; ++b) {
        const float* X = bq + (QS + 0 * 3 + b) * BN;
        const float* Y = bq + (QS + 1 * 3 + b) * BN;
        const float* Z = bq + (QS + 2 * 3 + b) * BN;
        const float xr = fmaf(4.f, X[1], X[-BW + 1] + X[BW + 1]) - fmaf(4.f, X[-1], X[-BW - 1] + X[BW - 1]);
        const float yr = fmaf(4.f, Y[BW] - Y[-BW], (Y[BW - 1] - Y[-BW - 1]) + (Y[BW + 1] - Y[-BW + 1]));
        const float t0 = fmaf(4.f, Z[-1], Z[-BW - 1] + Z[BW - 1]);
        const float t1 = fmaf(4.f, Z[0], Z[-BW] + Z[BW]);
        const float t2 = fmaf(4.f, Z[1], Z[-BW + 1] + Z[BW + 1]);
        const float zr = fmaf(4.f, t1, t0 + t2);
        const float Q = xr + yr;
        dv[b] = sk.d * (rD1[b] + Q + zr);
        rD1[b] = fmaf(4.f, Q, rD2[b]);
        rD2[b] = Q - zr;
      }
      if (i >= 4) {
        const int zc = z0 - 4 + i;
        const float* pq = sQ + ((i + 1) & 1) * 7 * CN;        // plane c, stage 1 + velocity terms
        const float* uc = sU + ((i + RU - 1) % RU) * 3 * BN;  // u at plane c
        const float* ac = sA + ((i + RA - 2) % RA) * 4 * AN;  // phi, P at plane c
        const int c = qy * TX + qx, oa = (qy + 2) * AW + (qx + 2);
        const size_t g = (size_t)zc * NN + gc;
        // u*_b = u_b + dt d/dt u_b (:480-482)
#pragma unroll
        for (int b = 0; b < 3; ++b) oUs[b][g] = uc[b * BN + qo] + p.dt * (pq[(PU + b) * CN + c] + dv[b]);
        // P*_b = P_b + dt (pointwise part + eta L mu_b) (:623-629, :486-488)
#pragma unroll
        for (int b = 0; b < 3; ++b) oPs[b][g] = ac[(1 + b) * AN + oa] + p.dt * (pq[(PP + b) * CN + c] + p.eta * lmu[b]);
        // phi' = phi + dt (-u.D phi + gamma L mu_0) (:631, :515), compensated: the part of the
        // increment that rounding drops from phi is carried to the next step (otherwise
        // increments below half an ulp of phi are lost, a systematic mass drift)
        const float ph = ac[oa];
        const float inc = fmaf(p.dt, pq[PPHI * CN + c] + p.gamma * lmu[3], cprev);
        const float nv = ph + inc;
        phic[g] = inc - (nv - ph);
        ophi[g] = nv;
      }
    }
  }
}

// ------------------------------------------------------------------------------------------
// fused_div / fused_correct: one tile column per thread; each staged plane is read once, its
// in-plane partial sums carried in z (as in fused_rhs phase 2), so the ring only has to cover
// the copies in flight: DR slots, the plane read and DR - 1 planes in flight. Rows are staged in
// 16-byte chunks: a row starts at a multiple of 4 floats (2 float2) left of the tile, so every
// chunk, wrapped or not, is one aligned 16-byte global segment (N is a multiple of 32).
constexpr int NTC = TX * TY;            // 512 threads
constexpr int SH = TY + 2;              // staged rows y0 - 1 .. y0 + TY
constexpr int SW = TX + 8;              // fused_div row, floats x0 - 4 .. x0 + TX + 3
constexpr int SPL = SW * SH;            // floats per staged plane of one field
constexpr int CW = TX + 4;              // fused_correct row, float2 x0 - 2 .. x0 + TX + 1
constexpr int CPL = CW * SH;            // float2 per staged plane
constexpr int DR = 4;                   // ring slots of fused_div / fused_correct
constexpr size_t DIV_SMEM = DR * 6 * SPL * sizeof(float);
constexpr size_t COR_SLOT = CPL * sizeof(float2) + 6 * CN * sizeof(float);  // p_v, p_p on B; u*, P* on C
constexpr size_t COR_SMEM = DR * COR_SLOT;

// wait until at most DR - 2 copy groups are pending: the group of the plane read now is complete
__device__ __forceinline__ void cp_async_wait_ring() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(DR - 2) : "memory");
}

__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem) : "memory");
}

__global__ void __launch_bounds__(NTC, 2) k_fused_div(const InstDev<float>* __restrict__ insts, int par, int nchunk) {
  extern __shared__ __align__(16) float sm[];
  const int N = insts[0].N;
  const InstDev<float>& I = insts[blockIdx.z / nchunk];
  const int x0 = blockIdx.x * TX, y0 = blockIdx.y * TY;
  const int z0 = (blockIdx.z % nchunk) * ZC, z1 = min(z0 + ZC, N);
  const size_t NN = (size_t)N * N;
  const float* cur[6] = {I.Us[par ^ 1][0], I.Us[par ^ 1][1], I.Us[par ^ 1][2],
                         I.Ps[par ^ 1][0], I.Ps[par ^ 1][1], I.Ps[par ^ 1][2]};
  const float* old[6] = {I.Us[par][0], I.Us[par][1], I.Us[par][2], I.Ps[par][0], I.Ps[par][1], I.Ps[par][2]};
  float2* const oW = I.W;
  const int stale_q2 = I.stale;
  const float kd = I.ph.c2h * (1.f / 36.f) * I.ph.inv_dt;  // d/36 of the 27-point D, and 1/dt
  const int tid = threadIdx.x;
  const int niter = (z1 - z0) + 2;
  // issue(i): plane z0 - 1 + i into slot i % DR (an empty group past the last plane, so that
  // every iteration commits one). Chunks outside the domain come from the previous step's u*, P*
  // when the stale-halo quirk is on (the chunk grid is aligned with 0 and N).
  auto issue = [&](int i) {
    if (i >= niter) { cp_async_commit(); return; }
    const int zu = z0 - 1 + i;
    const bool zw = zu < 0 || zu >= N;
    const int zz = wrapN(zu, N);
    float* dst = sm + (i % DR) * 6 * SPL;
    constexpr int CR = SW / 4;  // chunks per row
    for (int t = tid; t < SH * CR; t += NTC) {
      const int ry = t / CR, rc = t - ry * CR;
      const int gx = x0 - 4 + 4 * rc, gy = y0 - 1 + ry;
      const bool stale = stale_q2 && (zw || gx < 0 || gx >= N || gy < 0 || gy >= N);
      const size_t g = (size_t)zz * NN + (size_t)wrapN(gy, N) * N + wrapN(gx, N);
#pragma unroll
      for (int f = 0; f < 6; ++f) cp_async16(dst + f * SPL + ry * SW + 4 * rc, (stale ? old[f] : cur[f]) + g);
    }
    cp_async_commit();
  };
  const int qx = tid % TX, qy = tid / TX;
  const size_t gc = (size_t)(y0 + qy) * N + (x0 + qx);
  // the divergence D_x v_x + D_y v_y + D_z v_z of v = u*, P* (getStream mode 0, :664-670), each
  // D = d/36 delta s s: a plane adds Q = delta_x s_y v_x + s_x delta_y v_y with weight s_z =
  // (1, 4, 1) and Z = s_x s_y v_z with weight delta_z = (-1, 0, 1) over planes c-1, c, c+1
  float rD1[2] = {0.f, 0.f}, rD2[2] = {0.f, 0.f};
#pragma unroll
  for (int k = 0; k < DR - 1; ++k) issue(k);
  for (int i = 0; i < niter; ++i) {
    cp_async_wait_ring();
    __syncthreads();
    issue(i + DR - 1);  // into the slot read at iteration i - 1
    const float* s = sm + (i % DR) * 6 * SPL + (qy + 1) * SW + (qx + 4);
    float dv[2];
#pragma unroll
    for (int f = 0; f < 2; ++f) {
      const float* X = s + (3 * f + 0) * SPL;
      const float* Y = s + (3 * f + 1) * SPL;
      const float* Z = s + (3 * f + 2) * SPL;
      const float xr = fmaf(4.f, X[1], X[-SW + 1] + X[SW + 1]) - fmaf(4.f, X[-1], X[-SW - 1] + X[SW - 1]);
      const float yr = fmaf(4.f, Y[SW] - Y[-SW], (Y[SW - 1] - Y[-SW - 1]) + (Y[SW + 1] - Y[-SW + 1]));
      const float t0 = fmaf(4.f, Z[-1], Z[-SW - 1] + Z[SW - 1]);
      const float t1 = fmaf(4.f, Z[0], Z[-SW] + Z[SW]);
      const float t2 = fmaf(4.f, Z[1], Z[-SW + 1] + Z[SW + 1]);
      const float zr = fmaf(4.f, t1, t0 + t2);
      const float Q = xr + yr;
      dv[f] = rD1[f] + Q + zr;
      rD1[f] = fmaf(4.f, Q, rD2[f]);
      rD2[f] = Q - zr;
    }
    if (i >= 2) oW[(size_t)(z0 - 2 + i) * NN + gc] = make_float2(kd * dv[0], kd * dv[1]);
  }
}

__global__ void __launch_bounds__(NTC, 2) k_fused_correct(const InstDev<float>* __restrict__ insts, int par, int nchunk) {
  extern __shared__ __align__(16) unsigned char smc[];
  const int N = insts[0].N;
  const InstDev<float>& I = insts[blockIdx.z / nchunk];
  const float kd = I.ph.c2h * (1.f / 36.f);
  const float dt = I.ph.dt;
  const int x0 = blockIdx.x * TX, y0 = blockIdx.y * TY;
  const int z0 = (blockIdx.z % nchunk) * ZC, z1 = min(z0 + ZC, N);
  const size_t NN = (size_t)N * N;
  const int niter = (z1 - z0) + 2;
  const float* qs[6] = {I.Us[par ^ 1][0], I.Us[par ^ 1][1], I.Us[par ^ 1][2],
                        I.Ps[par ^ 1][0], I.Ps[par ^ 1][1], I.Ps[par ^ 1][2]};
  float* const oU[3] = {I.U[0], I.U[1], I.U[2]};
  float* const oP[3] = {I.P[0], I.P[1], I.P[2]};
  const float2* __restrict__ gW = I.W;
  const int tid = threadIdx.x;
  auto slot_w = [&](int i) { return reinterpret_cast<float2*>(smc + (i % DR) * COR_SLOT); };
  auto slot_q = [&](int i) { return reinterpret_cast<float*>(smc + (i % DR) * COR_SLOT + CPL * sizeof(float2)); };
  // issue(i): into slot i % DR the pressures (p_v, p_p) of plane z0 - 1 + i over tile+1 and u*, P*
  // of plane z0 - 2 + i (finished at iteration i) over the tile; an empty group past the last plane
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
      float* dq = slot_q(i);
      // 4 groups of TY * TX / 4 threads, one chunk of a tile row each: group k copies fields k, k + 4
      constexpr int QR = TX / 4, QG = TY * QR;  // chunks per tile row, per field
      static_assert(4 * QG == NTC, "chunk groups cover the block");
      const int r = tid % QG, fg = tid / QG;
      const int ry = r / QR, rc = r - ry * QR;
      const size_t go = (size_t)zq * NN + (size_t)(y0 + ry) * N + x0 + 4 * rc;
#pragma unroll
      for (int f = 0; f < 6; ++f)
        if ((f & 3) == fg) cp_async16(dq + f * CN + ry * TX + 4 * rc, qs[f] + go);
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
      const float* qc = slot_q(i) + qy * TX + qx;
      const float gv[3] = {gx.x, gy.x, gz.x}, gp[3] = {gx.y, gy.y, gz.y};
#pragma unroll
      for (int b = 0; b < 3; ++b) {
        oU[b][g] = qc[b * CN] - dt * (kd * gv[b]);
        oP[b][g] = qc[(3 + b) * CN] - dt * (kd * gp[b]);
      }
    }
  }
}

inline void check(cudaError_t e, const char* what) {
  if (e != cudaSuccess) throw std::runtime_error(std::string(what) + ": " + cudaGetErrorString(e));
}

dim3 grid_for(const Group<float>& g, int& nchunk) {
  nchunk = (g.N + ZC - 1) / ZC;
  if ((long)nchunk * g.n > 65535) throw std::runtime_error("fused: too many droplets in one group");
  return dim3(g.N / TX, g.N / TY, nchunk * g.n);
}

}  // namespace

bool fused_supported(int N) { return N >= 32 && N % TX == 0 && N % TY == 0; }

void fused_prepare() {
  check(cudaFuncSetAttribute(k_fused_rhs, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)RHS_SMEM),
        "fused_rhs smem attribute");
  check(cudaFuncSetAttribute(k_fused_div, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)DIV_SMEM),
        "fused_div smem attribute");
  check(cudaFuncSetAttribute(k_fused_correct, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)COR_SMEM),
        "fused_correct smem attribute");
}

void launch_fused_rhs(const Group<float>& g, int par, cudaStream_t st) {
  int nchunk;
  dim3 grid = grid_for(g, nchunk);
  k_fused_rhs<<<grid, NT, RHS_SMEM, st>>>(g.d_inst, par, nchunk);
  check(cudaGetLastError(), "fused_rhs launch");
}

void launch_fused_div(const Group<float>& g, int par, cudaStream_t st) {
  int nchunk;
  dim3 grid = grid_for(g, nchunk);
  k_fused_div<<<grid, NTC, DIV_SMEM, st>>>(g.d_inst, par, nchunk);
  check(cudaGetLastError(), "fused_div launch");
}

void launch_fused_correct(const Group<float>& g, int par, cudaStream_t st) {
  int nchunk;
  dim3 grid = grid_for(g, nchunk);
  k_fused_correct<<<grid, NTC, COR_SMEM, st>>>(g.d_inst, par, nchunk);
  check(cudaGetLastError(), "fused_correct launch");
}

}  // namespace ttsh
