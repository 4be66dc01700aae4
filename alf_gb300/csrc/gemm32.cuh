// Batched complex GEMM in double-float arithmetic on the FP32 pipes (the mixed form).
//
// Each FP64 operand element is split into an unevaluated sum hi + lo of two
// floats (hi = fl32(x), lo = fl32(x - hi)); products use the exact FMA
// two-product and are accumulated with a two-sum, so a dot product carries a
// ~2^-44 relative rounding instead of FP32's 2^-24.  On GB300 the FP32 pipes
// run 64x the FP64 rate (66 vs 1.0 TFLOP/s measured); a double-float
// multiply-accumulate costs ~14 FP32 operations.  Same operation and options
// as k_zgemm (gemm.cuh); operands and output may be stored as complex128 or
// real64.  The FP32 exponent range (|x| < 3.4e38) suffices for the G wraps and
// flushes (|G_ij| = O(1), |expT| = O(1)); the graded UDV products stay FP64.
#pragma once
#include "gemm.cuh"

enum { ST_C128 = 0, ST_R64 = 2 };

struct Gemm32Params {
  GemmParams g;   // sizes, strides (in elements), ops, masks, scales, permutations; realA/realB ignored
  int tA, tB, tC; // storage types (ST_*)
};

struct dfc {      // complex double-float: re = rh + rl, im = ih + il
  float rh, rl, ih, il;
};

ALF_DEV void df_split(double x, float& h, float& l) {
  h = __double2float_rn(x);
  l = __double2float_rn(x - (double)h);
}
ALF_DEV dfc dfc_ld(const void* X, int st, long long idx) {
  dfc r;
  if (st == ST_C128) {
    const double2 v = ((const double2*)X)[idx];
    df_split(v.x, r.rh, r.rl);
    df_split(v.y, r.ih, r.il);
  } else {
    df_split(((const double*)X)[idx], r.rh, r.rl);
    r.ih = 0.f; r.il = 0.f;
  }
  return r;
}
// acc += a * b (double-float, Dekker two-product with FMA, two-sum accumulation)
ALF_DEV void df_mac(float& ah, float& al, float xh, float xl, float yh, float yl) {
  const float p = xh * yh;
  float e = fmaf(xh, yh, -p);
  e = fmaf(xh, yl, e);
  e = fmaf(xl, yh, e);
  const float s = ah + p;
  const float bb = s - ah;
  float t = (ah - (s - bb)) + (p - bb);
  t += al + e;
  ah = s + t;
  al = t - (ah - s);
}

// BM x BN tile, 256 threads as 16 x 16, each thread (BM/16) x (BN/16) outputs.
template <int BM, int BN>
__global__ void __launch_bounds__(256) k_dfgemm(Gemm32Params P) {
  constexpr int BK = 8, TM = BM / 16, TN = BN / 16;
  __shared__ dfc As[BK][BM + 1];
  __shared__ dfc Bs[BK][BN + 1];
  const GemmParams& p = P.g;
  const int b = blockIdx.z;
  const int m0 = blockIdx.y * BM, n0 = blockIdx.x * BN;
  const int tid = threadIdx.x, tx = tid % 16, ty = tid / 16;
  const int K = p.kdyn ? min(p.kdyn[b], p.k) : p.k;
  const int bA = p.modA > 0 ? b % p.modA : b, bB = p.modB > 0 ? b % p.modB : b;
  const size_t szA = P.tA == ST_C128 ? 16 : 8, szB = P.tB == ST_C128 ? 16 : 8;
  const char* A = (const char*)p.A + (size_t)bA * p.sA * szA;
  const char* B = (const char*)p.B + (size_t)bB * p.sB * szB;
  const zd* ks = p.ks ? p.ks + b * p.sKS : nullptr;
  const int* pA = p.permA ? p.permA + b * p.sPA : nullptr;
  const int* pB = p.permB ? p.permB + b * p.sPB : nullptr;
  const bool cplxA = P.tA == ST_C128, cplxB = P.tB == ST_C128;
  const bool aImag = cplxA || (p.ks && p.ksOnA), bImag = cplxB || (p.ks && !p.ksOnA);
  float acc[TM][TN][4];
#pragma unroll
  for (int i = 0; i < TM; ++i)
#pragma unroll
    for (int j = 0; j < TN; ++j) acc[i][j][0] = acc[i][j][1] = acc[i][j][2] = acc[i][j][3] = 0.f;

  for (int k0 = 0; k0 < K; k0 += BK) {
    for (int e = tid; e < BM * BK; e += 256) {
      int i, kk;
      if (p.opA == OP_N) { i = e % BM; kk = e / BM; } else { kk = e % BK; i = e / BK; }
      const int gi = m0 + i, gk = k0 + kk;
      dfc v = {0.f, 0.f, 0.f, 0.f};
      if (gi < p.m && gk < K) {
        const int kq = pA ? pA[gk] : gk;
        long long r, c;
        if (p.opA == OP_N) { r = gi; c = kq; } else { r = kq; c = gi; }
        if (!(p.triA && r > c)) {
          if (ks && p.ksOnA) {  // scale in FP64 before the split
            zd x = cplxA ? ((const double2*)A)[r + c * p.lda] : zmk(((const double*)A)[r + c * p.lda], 0.0);
            if (p.opA == OP_C) x.y = -x.y;
            zd s = ks[gk];
            if (p.ksConj) s.y = -s.y;
            x = zmul(x, s);
            df_split(x.x, v.rh, v.rl);
            df_split(x.y, v.ih, v.il);
          } else {
            v = dfc_ld(A, P.tA, r + c * p.lda);
            if (p.opA == OP_C) { v.ih = -v.ih; v.il = -v.il; }
          }
        }
      }
      As[kk][i] = v;
    }
    for (int e = tid; e < BN * BK; e += 256) {
      int j, kk;
      if (p.opB == OP_N) { kk = e % BK; j = e / BK; } else { j = e % BN; kk = e / BN; }
      const int gj = n0 + j, gk = k0 + kk;
      dfc v = {0.f, 0.f, 0.f, 0.f};
      if (gj < p.n && gk < K) {
        const int kq = pB ? pB[gk] : gk;
        long long r, c;
        if (p.opB == OP_N) { r = kq; c = gj; } else { r = gj; c = kq; }
        if (!(p.triB && r > c)) {
          if (ks && !p.ksOnA) {
            zd x = cplxB ? ((const double2*)B)[r + c * p.ldb] : zmk(((const double*)B)[r + c * p.ldb], 0.0);
            if (p.opB == OP_C) x.y = -x.y;
            zd s = ks[gk];
            if (p.ksConj) s.y = -s.y;
            x = zmul(x, s);
            df_split(x.x, v.rh, v.rl);
            df_split(x.y, v.ih, v.il);
          } else {
            v = dfc_ld(B, P.tB, r + c * p.ldb);
            if (p.opB == OP_C) { v.ih = -v.ih; v.il = -v.il; }
          }
        }
      }
      Bs[kk][j] = v;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < BK; ++kk) {
      dfc a[TM], bb[TN];
#pragma unroll
      for (int i = 0; i < TM; ++i) a[i] = As[kk][ty + 16 * i];
#pragma unroll
      for (int j = 0; j < TN; ++j) bb[j] = Bs[kk][tx + 16 * j];
#pragma unroll
      for (int i = 0; i < TM; ++i)
#pragma unroll
        for (int j = 0; j < TN; ++j) {
          float* c = acc[i][j];
          df_mac(c[0], c[1], a[i].rh, a[i].rl, bb[j].rh, bb[j].rl);                  // re += ar br
          if (bImag) df_mac(c[2], c[3], a[i].rh, a[i].rl, bb[j].ih, bb[j].il);        // im += ar bi
          if (aImag) df_mac(c[2], c[3], a[i].ih, a[i].il, bb[j].rh, bb[j].rl);        // im += ai br
          if (aImag && bImag) df_mac(c[0], c[1], -a[i].ih, -a[i].il, bb[j].ih, bb[j].il);  // re -= ai bi
        }
    }
    __syncthreads();
  }
  const zd* rs = p.rs ? p.rs + b * p.sRS : nullptr;
  const zd* cs = p.cs ? p.cs + b * p.sCS : nullptr;
  const bool usebeta = (p.beta.x != 0.0 || p.beta.y != 0.0);
  double2* C = (double2*)p.C + (size_t)b * p.sC;
#pragma unroll
  for (int i = 0; i < TM; ++i)
#pragma unroll
    for (int j = 0; j < TN; ++j) {
      const int row = m0 + ty + 16 * i, col = n0 + tx + 16 * j;
      if (row >= p.m || col >= p.n) continue;
      zd v = zmk((double)acc[i][j][0] + (double)acc[i][j][1], (double)acc[i][j][2] + (double)acc[i][j][3]);
      if (rs) v = p.rsInv ? zdiv(v, rs[row]) : zmul(rs[row], v);
      if (cs) v = p.csInv ? zdiv(v, cs[col]) : zmul(v, cs[col]);
      v = zmul(p.alpha, v);
      double2* cp = C + row + (long long)col * p.ldc;
      if (usebeta) v = zadd(v, zmul(p.beta, *cp));
      *cp = v;
    }
}

static inline cudaError_t launch_dfgemm(const Gemm32Params& P, cudaStream_t st) {
  const GemmParams& p = P.g;
  if (p.m <= 0 || p.n <= 0 || p.batch <= 0) return cudaSuccess;
  long long tiles64 = (long long)((p.m + 63) / 64) * ((p.n + 63) / 64) * p.batch;
  if (tiles64 >= 256) {
    dim3 grid((p.n + 63) / 64, (p.m + 63) / 64, p.batch);
    k_dfgemm<64, 64><<<grid, 256, 0, st>>>(P);
  } else {
    dim3 grid((p.n + 31) / 32, (p.m + 31) / 32, p.batch);
    k_dfgemm<32, 32><<<grid, 256, 0, st>>>(P);
  }
  return cudaGetLastError();
}
