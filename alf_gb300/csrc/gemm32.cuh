// Batched complex GEMM computed in FP32 (the complex64 arithmetic of the mixed
// form).  Same operation and options as k_zgemm (gemm.cuh); each operand and the
// output may be stored as complex128, complex64, real64 or real32, so the FP64
// state of the stabilisation (U, V) and the complex64 G of the mixed sweep can be
// fed without conversion passes.
#pragma once
#include "gemm.cuh"

enum { ST_C128 = 0, ST_C64 = 1, ST_R64 = 2, ST_R32 = 3 };

struct Gemm32Params {
  GemmParams g;   // sizes, strides (in elements), ops, masks, scales, permutations; realA/realB ignored
  int tA, tB, tC; // storage types (ST_*)
};

ALF_DEV float2 ld_any(const void* X, int st, long long idx) {
  switch (st) {
    case ST_C128: { double2 v = ((const double2*)X)[idx]; return make_float2((float)v.x, (float)v.y); }
    case ST_C64: return ((const float2*)X)[idx];
    case ST_R64: return make_float2((float)((const double*)X)[idx], 0.f);
    default: return make_float2(((const float*)X)[idx], 0.f);
  }
}
ALF_HD size_t st_size(int st) { return st == ST_C128 ? 16 : (st == ST_C64 || st == ST_R64) ? 8 : 4; }

ALF_DEV float2 cmulf(float2 a, float2 b) { return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x); }

// BM x BN tile, 256 threads as 16 x 16, each thread (BM/16) x (BN/16) outputs.
template <int BM, int BN>
__global__ void __launch_bounds__(256) k_cgemm32(Gemm32Params P) {
  constexpr int BK = 16, TM = BM / 16, TN = BN / 16;
  __shared__ float2 As[BK][BM + 1];
  __shared__ float2 Bs[BK][BN + 1];
  const GemmParams& p = P.g;
  const int b = blockIdx.z;
  const int m0 = blockIdx.y * BM, n0 = blockIdx.x * BN;
  const int tid = threadIdx.x, tx = tid % 16, ty = tid / 16;
  const int K = p.kdyn ? min(p.kdyn[b], p.k) : p.k;
  const int bA = p.modA > 0 ? b % p.modA : b, bB = p.modB > 0 ? b % p.modB : b;
  const char* A = (const char*)p.A + (size_t)bA * p.sA * st_size(P.tA);
  const char* B = (const char*)p.B + (size_t)bB * p.sB * st_size(P.tB);
  const zd* ks = p.ks ? p.ks + b * p.sKS : nullptr;
  const int* pA = p.permA ? p.permA + b * p.sPA : nullptr;
  const int* pB = p.permB ? p.permB + b * p.sPB : nullptr;
  float2 acc[TM][TN];
#pragma unroll
  for (int i = 0; i < TM; ++i)
#pragma unroll
    for (int j = 0; j < TN; ++j) acc[i][j] = make_float2(0.f, 0.f);

  for (int k0 = 0; k0 < K; k0 += BK) {
    for (int e = tid; e < BM * BK; e += 256) {
      int i, kk;
      if (p.opA == OP_N) { i = e % BM; kk = e / BM; } else { kk = e % BK; i = e / BK; }
      const int gi = m0 + i, gk = k0 + kk;
      float2 v = make_float2(0.f, 0.f);
      if (gi < p.m && gk < K) {
        const int kq = pA ? pA[gk] : gk;
        long long r, c;
        if (p.opA == OP_N) { r = gi; c = kq; } else { r = kq; c = gi; }
        if (!(p.triA && r > c)) {
          v = ld_any(A, P.tA, r + c * p.lda);
          if (p.opA == OP_C) v.y = -v.y;
        }
        if (ks && p.ksOnA) {
          zd s = ks[gk];
          if (p.ksConj) s.y = -s.y;
          v = cmulf(v, make_float2((float)s.x, (float)s.y));
        }
      }
      As[kk][i] = v;
    }
    for (int e = tid; e < BN * BK; e += 256) {
      int j, kk;
      if (p.opB == OP_N) { kk = e % BK; j = e / BK; } else { j = e % BN; kk = e / BN; }
      const int gj = n0 + j, gk = k0 + kk;
      float2 v = make_float2(0.f, 0.f);
      if (gj < p.n && gk < K) {
        const int kq = pB ? pB[gk] : gk;
        long long r, c;
        if (p.opB == OP_N) { r = kq; c = gj; } else { r = gj; c = kq; }
        if (!(p.triB && r > c)) {
          v = ld_any(B, P.tB, r + c * p.ldb);
          if (p.opB == OP_C) v.y = -v.y;
        }
        if (ks && !p.ksOnA) {
          zd s = ks[gk];
          if (p.ksConj) s.y = -s.y;
          v = cmulf(v, make_float2((float)s.x, (float)s.y));
        }
      }
      Bs[kk][j] = v;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < BK; ++kk) {
      float2 a[TM], bb[TN];
#pragma unroll
      for (int i = 0; i < TM; ++i) a[i] = As[kk][ty + 16 * i];
#pragma unroll
      for (int j = 0; j < TN; ++j) bb[j] = Bs[kk][tx + 16 * j];
#pragma unroll
      for (int i = 0; i < TM; ++i)
#pragma unroll
        for (int j = 0; j < TN; ++j) {
          acc[i][j].x = fmaf(a[i].x, bb[j].x, acc[i][j].x);
          acc[i][j].x = fmaf(-a[i].y, bb[j].y, acc[i][j].x);
          acc[i][j].y = fmaf(a[i].x, bb[j].y, acc[i][j].y);
          acc[i][j].y = fmaf(a[i].y, bb[j].x, acc[i][j].y);
        }
    }
    __syncthreads();
  }
  const zd* rs = p.rs ? p.rs + b * p.sRS : nullptr;
  const zd* cs = p.cs ? p.cs + b * p.sCS : nullptr;
  const bool usebeta = (p.beta.x != 0.0 || p.beta.y != 0.0);
  char* C = (char*)p.C + (size_t)b * p.sC * st_size(P.tC);
#pragma unroll
  for (int i = 0; i < TM; ++i)
#pragma unroll
    for (int j = 0; j < TN; ++j) {
      const int row = m0 + ty + 16 * i, col = n0 + tx + 16 * j;
      if (row >= p.m || col >= p.n) continue;
      float2 v = acc[i][j];
      if (rs) { zd s = rs[row]; v = cmulf(make_float2((float)s.x, (float)s.y), v); }
      if (cs) { zd s = cs[col]; v = cmulf(v, make_float2((float)s.x, (float)s.y)); }
      v = cmulf(make_float2((float)p.alpha.x, (float)p.alpha.y), v);
      const long long idx = row + (long long)col * p.ldc;
      if (P.tC == ST_C64) {
        float2* cp = (float2*)C + idx;
        if (usebeta) v = make_float2(v.x + (float)p.beta.x * cp->x - (float)p.beta.y * cp->y,
                                     v.y + (float)p.beta.x * cp->y + (float)p.beta.y * cp->x);
        *cp = v;
      } else {
        double2* cp = (double2*)C + idx;
        zd w = zmk((double)v.x, (double)v.y);
        if (usebeta) w = zadd(w, zmul(p.beta, *cp));
        *cp = w;
      }
    }
}

static inline cudaError_t launch_cgemm32(const Gemm32Params& P, cudaStream_t st) {
  const GemmParams& p = P.g;
  if (p.m <= 0 || p.n <= 0 || p.batch <= 0) return cudaSuccess;
  long long tiles64 = (long long)((p.m + 63) / 64) * ((p.n + 63) / 64) * p.batch;
  if (tiles64 >= 256) {
    dim3 grid((p.n + 63) / 64, (p.m + 63) / 64, p.batch);
    k_cgemm32<64, 64><<<grid, 256, 0, st>>>(P);
  } else {
    dim3 grid((p.n + 31) / 32, (p.m + 31) / 32, p.batch);
    k_cgemm32<32, 32><<<grid, 256, 0, st>>>(P);
  }
  return cudaGetLastError();
}

// float2 <-> double2 conversion of batched matrices
__global__ void k_c128_to_c64(const double2* in, float2* out, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    out[i] = make_float2((float)in[i].x, (float)in[i].y);
}
__global__ void k_c64_to_c128(const float2* in, double2* out, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    out[i] = zmk((double)in[i].x, (double)in[i].y);
}
// G(i,j) <- S(i) G(i,j) Sinv(j) on complex64 storage
__global__ void k_apply_scale32(float2* G, const zd* S, const zd* Sinv, int N) {
  const int b = blockIdx.y;
  const long long NN = (long long)N * N;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < NN; e += (long long)gridDim.x * blockDim.x) {
    const int i = e % N, j = e / N;
    float2* g = G + b * NN + e;
    const zd s = S[(long long)b * N + i], si = Sinv[(long long)b * N + j];
    *g = cmulf(cmulf(make_float2((float)s.x, (float)s.y), *g), make_float2((float)si.x, (float)si.y));
  }
}
