// Batched complex128 GEMM on the FP64 tensor path (mma.sync m8n8k4 f64, DMMA).
//
//   C = alpha * rs .* ( op(A) * diag(ks) * op(B) ) .* cs + beta * C
//
// with op in {N, T, C}, either operand optionally real (the ZLARCM/ZLACRM case
// of ALF's dense hopping products, Libraries/Modules/Mat_subroutines_mod.F90:1225-1418),
// an optional K-dimension gather on either operand (ZLAPMR/ZLAPMT row/column
// permutations folded into the load), an optional "stored upper triangular"
// mask (ZTRMM with R kept above the Householder vectors), per-batch K read from
// device memory (delayed-update flushes whose rank differs per chain), and a
// row/column scaling epilogue (the D scalings of CGR, Prog/cgr1_mod.F90:233-236).
#pragma once
#include "common.cuh"

enum { OP_N = 0, OP_T = 1, OP_C = 2 };

struct GemmParams {
  int m, n, k;
  const void* A; long long lda, sA; int opA, realA, triA;
  const void* B; long long ldb, sB; int opB, realB, triB;
  zd* C; long long ldc, sC;
  zd alpha, beta;
  const zd* ks; long long sKS; int ksOnA, ksConj, ksInv;
  const zd* rs; long long sRS; int rsInv;
  const zd* cs; long long sCS; int csInv;
  const int* permA; long long sPA;
  const int* permB; long long sPB;
  const int* kdyn;  // per-batch K (<= k) or null
  int batch;
  int modA, modB;   // if > 0, operand batch index = b % mod (an operand shared across chains)
  int ksplit;       // > 1: K split over ksplit CTAs per tile, partials into ws, summed by k_zgemm_reduce
  zd* ws;           // [ksplit][batch][m][n] partial products (column-major per matrix)
};

static inline GemmParams gemm_defaults() {
  GemmParams p;
  memset(&p, 0, sizeof(p));
  p.alpha = zmk(1.0, 0.0);
  p.beta = zmk(0.0, 0.0);
  p.batch = 1;
  p.ksplit = 1;
  return p;
}

#define GEMM_BK 16

ALF_DEV void dmma(double& d0, double& d1, double a, double b) {
  asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0,%1}, {%2}, {%3}, {%0,%1};"
               : "+d"(d0), "+d"(d1)
               : "d"(a), "d"(b));
}

// Load op(X)(i, kk) of one operand (global), returning complex.
ALF_DEV zd gemm_ld(const void* X, long long ld, int op, int isreal, int tri, const int* perm, int i, int kk,
                   int rows, int kmax) {
  if (i >= rows || kk >= kmax) return zmk(0.0, 0.0);
  int kq = perm ? perm[kk] : kk;
  long long r, c;
  if (op == OP_N) { r = i; c = kq; } else { r = kq; c = i; }
  if (tri && r > c) return zmk(0.0, 0.0);
  zd v;
  if (isreal) v = zmk(((const double*)X)[r + c * ld], 0.0);
  else v = ((const zd*)X)[r + c * ld];
  if (op == OP_C) v.y = -v.y;
  return v;
}

// BM x BN tile per CTA, warps of WM x 16.
template <int BM, int BN, int WM>
__global__ void __launch_bounds__((BM / WM) * (BN / 16) * 32) k_zgemm(GemmParams p) {
  constexpr int WN = 16;
  constexpr int WARPS_M = BM / WM, WARPS_N = BN / WN;
  constexpr int NT = WARPS_M * WARPS_N * 32;
  constexpr int MI = WM / 8, NI = WN / 8;
  constexpr int SA = BM + 4, SB = BN + 4;
  __shared__ double As[2][GEMM_BK][SA];  // [re/im][k][m]
  __shared__ double Bs[2][GEMM_BK][SB];  // [re/im][k][n]

  const int ksplit = p.ksplit > 1 ? p.ksplit : 1;
  const int b = blockIdx.z / ksplit, sidx = blockIdx.z % ksplit;
  const int m0 = blockIdx.y * BM, n0 = blockIdx.x * BN;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int wm = (warp % WARPS_M) * WM, wn = (warp / WARPS_M) * WN;
  const int g = lane >> 2, t = lane & 3;

  const int Kall = p.kdyn ? min(p.kdyn[b], p.k) : p.k;
  // this CTA's K range (split-K): chunks of whole k-tiles
  const int kchunk = ((p.k + ksplit - 1) / ksplit + GEMM_BK - 1) / GEMM_BK * GEMM_BK;
  const int kbeg = sidx * kchunk;
  const int K = min(Kall, kbeg + kchunk);
  const int bA = p.modA > 0 ? b % p.modA : b, bB = p.modB > 0 ? b % p.modB : b;
  const void* A = p.realA ? (const void*)((const double*)p.A + bA * p.sA) : (const void*)((const zd*)p.A + bA * p.sA);
  const void* B = p.realB ? (const void*)((const double*)p.B + bB * p.sB) : (const void*)((const zd*)p.B + bB * p.sB);
  zd* C = p.C + b * p.sC;
  const zd* ks = p.ks ? p.ks + b * p.sKS : nullptr;
  const int* pA = p.permA ? p.permA + b * p.sPA : nullptr;
  const int* pB = p.permB ? p.permB + b * p.sPB : nullptr;
  const bool cplx = !(p.realA || p.realB);

  double acc[MI][NI][2][2];
#pragma unroll
  for (int i = 0; i < MI; ++i)
#pragma unroll
    for (int j = 0; j < NI; ++j) acc[i][j][0][0] = acc[i][j][0][1] = acc[i][j][1][0] = acc[i][j][1][1] = 0.0;

  constexpr int AE = BM * GEMM_BK / NT;  // elements per thread
  constexpr int BE = BN * GEMM_BK / NT;
  zd ra[AE], rb[BE];

  auto load_tile = [&](int k0) {
#pragma unroll
    for (int r = 0; r < AE; ++r) {
      int e = tid + r * NT, i, kk;
      if (p.opA == OP_N) { i = e % BM; kk = e / BM; } else { kk = e % GEMM_BK; i = e / GEMM_BK; }
      zd v = gemm_ld(A, p.lda, p.opA, p.realA, p.triA, pA, m0 + i, k0 + kk, p.m, K);  // K: end of this range
      if (ks && p.ksOnA && k0 + kk < K) {
        zd s = ks[k0 + kk];
        if (p.ksConj) s.y = -s.y;
        v = p.ksInv ? zdiv(v, s) : zmul(v, s);
      }
      ra[r] = v;
    }
#pragma unroll
    for (int r = 0; r < BE; ++r) {
      int e = tid + r * NT, j, kk;
      if (p.opB == OP_N) { kk = e % GEMM_BK; j = e / GEMM_BK; } else { j = e % BN; kk = e / BN; }
      // op(B)(kk, j): stored (kk, j) for N, (j, kk) for T/C
      zd v;
      {
        int kq = k0 + kk, jj = n0 + j;
        if (kq >= K || jj >= p.n) v = zmk(0.0, 0.0);
        else {
          int kr = pB ? pB[kq] : kq;
          long long rr, cc;
          if (p.opB == OP_N) { rr = kr; cc = jj; } else { rr = jj; cc = kr; }
          if (p.triB && rr > cc) v = zmk(0.0, 0.0);
          else {
            if (p.realB) v = zmk(((const double*)B)[rr + cc * p.ldb], 0.0);
            else v = ((const zd*)B)[rr + cc * p.ldb];
            if (p.opB == OP_C) v.y = -v.y;
          }
          if (ks && !p.ksOnA) {
            zd s = ks[kq];
            if (p.ksConj) s.y = -s.y;
            v = p.ksInv ? zdiv(v, s) : zmul(v, s);
          }
        }
      }
      rb[r] = v;
    }
  };
  auto store_tile = [&]() {
#pragma unroll
    for (int r = 0; r < AE; ++r) {
      int e = tid + r * NT, i, kk;
      if (p.opA == OP_N) { i = e % BM; kk = e / BM; } else { kk = e % GEMM_BK; i = e / GEMM_BK; }
      As[0][kk][i] = ra[r].x;
      As[1][kk][i] = ra[r].y;
    }
#pragma unroll
    for (int r = 0; r < BE; ++r) {
      int e = tid + r * NT, j, kk;
      if (p.opB == OP_N) { kk = e % GEMM_BK; j = e / GEMM_BK; } else { j = e % BN; kk = e / BN; }
      Bs[0][kk][j] = rb[r].x;
      Bs[1][kk][j] = rb[r].y;
    }
  };

  const int nk = K > kbeg ? (K - kbeg + GEMM_BK - 1) / GEMM_BK : 0;
  if (nk > 0) load_tile(kbeg);
  for (int kt = 0; kt < nk; ++kt) {
    __syncthreads();
    store_tile();
    __syncthreads();
    if (kt + 1 < nk) load_tile(kbeg + (kt + 1) * GEMM_BK);
#pragma unroll
    for (int k4 = 0; k4 < GEMM_BK; k4 += 4) {
      double ar[MI], ai[MI], br[NI], bi[NI];
#pragma unroll
      for (int i = 0; i < MI; ++i) {
        ar[i] = As[0][k4 + t][wm + i * 8 + g];
        ai[i] = As[1][k4 + t][wm + i * 8 + g];
      }
#pragma unroll
      for (int j = 0; j < NI; ++j) {
        br[j] = Bs[0][k4 + t][wn + j * 8 + g];
        bi[j] = Bs[1][k4 + t][wn + j * 8 + g];
      }
      // the four real products of a complex tile, interleaved over the warp's tiles so that
      // consecutive MMAs never update the same accumulator
#pragma unroll
      for (int i = 0; i < MI; ++i)
#pragma unroll
        for (int j = 0; j < NI; ++j) dmma(acc[i][j][0][0], acc[i][j][0][1], ar[i], br[j]);
      if (!p.realB) {
#pragma unroll
        for (int i = 0; i < MI; ++i)
#pragma unroll
          for (int j = 0; j < NI; ++j) dmma(acc[i][j][1][0], acc[i][j][1][1], ar[i], bi[j]);
      }
      if (!p.realA) {
#pragma unroll
        for (int i = 0; i < MI; ++i)
#pragma unroll
          for (int j = 0; j < NI; ++j) dmma(acc[i][j][1][0], acc[i][j][1][1], ai[i], br[j]);
      }
      if (cplx) {
#pragma unroll
        for (int i = 0; i < MI; ++i)
#pragma unroll
          for (int j = 0; j < NI; ++j) dmma(acc[i][j][0][0], acc[i][j][0][1], -ai[i], bi[j]);
      }
    }
  }

  const zd* rs = p.rs ? p.rs + b * p.sRS : nullptr;
  const zd* cs = p.cs ? p.cs + b * p.sCS : nullptr;
  const bool usebeta = (p.beta.x != 0.0 || p.beta.y != 0.0);
#pragma unroll
  for (int i = 0; i < MI; ++i)
#pragma unroll
    for (int j = 0; j < NI; ++j)
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        int row = m0 + wm + i * 8 + g, col = n0 + wn + j * 8 + 2 * t + h;
        if (row < p.m && col < p.n) {
          zd v = zmk(acc[i][j][0][h], acc[i][j][1][h]);
          if (ksplit > 1) {  // raw partial; scalings and beta in k_zgemm_reduce
            p.ws[((long long)sidx * p.batch + b) * p.m * p.n + row + (long long)col * p.m] = v;
            continue;
          }
          if (rs) v = p.rsInv ? zdiv(v, rs[row]) : zmul(rs[row], v);
          if (cs) v = p.csInv ? zdiv(v, cs[col]) : zmul(v, cs[col]);
          v = zmul(p.alpha, v);
          zd* cp = C + row + (long long)col * p.ldc;
          if (usebeta) v = zadd(v, zmul(p.beta, *cp));
          *cp = v;
        }
      }
}

// C = alpha op(rs) (sum_s partial_s) op(cs) + beta C, partials summed in split order (deterministic).
// grid (ceil(m*n/256), batch)
__global__ void k_zgemm_reduce(GemmParams p) {
  const int b = blockIdx.y;
  const long long mn = (long long)p.m * p.n;
  const long long e = blockIdx.x * 256ll + threadIdx.x;
  if (e >= mn) return;
  const int row = e % p.m, col = e / p.m;
  zd v = p.ws[(long long)b * mn + e];
  for (int s = 1; s < p.ksplit; ++s) v = zadd(v, p.ws[((long long)s * p.batch + b) * mn + e]);
  const zd* rs = p.rs ? p.rs + b * p.sRS : nullptr;
  const zd* cs = p.cs ? p.cs + b * p.sCS : nullptr;
  if (rs) v = p.rsInv ? zdiv(v, rs[row]) : zmul(rs[row], v);
  if (cs) v = p.csInv ? zdiv(v, cs[col]) : zmul(v, cs[col]);
  v = zmul(p.alpha, v);
  zd* cp = p.C + b * p.sC + row + (long long)col * p.ldc;
  if (p.beta.x != 0.0 || p.beta.y != 0.0) v = zadd(v, zmul(p.beta, *cp));
  *cp = v;
}

// Host launcher: 64 x 64 tiles when there are enough of them; otherwise 32 x 32 tiles, and
// when even those leave SMs idle and K is long, K is split (workspace permitting) so that
// several CTAs per SM hide the latency between dependent FP64 MMAs.
static inline cudaError_t launch_zgemm(const GemmParams& p0, cudaStream_t st, zd* ws = nullptr,
                                       long long ws_elems = 0, int* nlaunch = nullptr) {
  GemmParams p = p0;
  p.ksplit = 1;
  if (nlaunch) *nlaunch = 1;
  if (p.m <= 0 || p.n <= 0 || p.batch <= 0) return cudaSuccess;
  long long tiles64 = (long long)((p.m + 63) / 64) * ((p.n + 63) / 64) * p.batch;
  if (tiles64 >= 256) {
    dim3 grid((p.n + 63) / 64, (p.m + 63) / 64, p.batch);
    k_zgemm<64, 64, 32><<<grid, 256, 0, st>>>(p);
    return cudaGetLastError();
  }
  const long long tiles32 = (long long)((p.n + 31) / 32) * ((p.m + 31) / 32) * p.batch;
  int ks = 1;
  while (ks < 4 && tiles32 * ks < 3 * 152 && p.k / (2 * ks) >= 64) ks *= 2;
  if (ks > 1 && ws && (long long)ks * p.batch * p.m * p.n <= ws_elems) {
    p.ksplit = ks;
    p.ws = ws;
  }
  dim3 grid((p.n + 31) / 32, (p.m + 31) / 32, p.batch * p.ksplit);
  k_zgemm<32, 32, 16><<<grid, 128, 0, st>>>(p);
  if (p.ksplit > 1) {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    dim3 rg((unsigned)(((long long)p.m * p.n + 255) / 256), p.batch);
    k_zgemm_reduce<<<rg, 256, 0, st>>>(p);
    if (nlaunch) *nlaunch = 2;
  }
  return cudaGetLastError();
}
