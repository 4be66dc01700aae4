// Time-displaced Green functions: TAU_M (Prog/tau_m_mod.F90:56-263) and the
// 2N x 2N block inversion CGR2_2, default branch (Prog/cgr2_2_mod.F90:55-73,
// 155-191, 317-425).  The propagations PROPR / PROPRM1 are scaled GEMMs issued by
// the host code; these kernels assemble and disassemble the block system and
// keep the precision statistics (Control_Precision_tau, control_mod.F90).
#pragma once
#include "common.cuh"

// G00 = GT0 = GTT = G, G0T = -(1 - G)  (tau_m_mod.F90:98-108).  grid (ceil(NN/256), B)
__global__ void k_tau_init(const zd* G, zd* G00, zd* GT0, zd* GTT, zd* G0T, int N) {
  const long long NN = (long long)N * N, b = blockIdx.y;
  const long long e = blockIdx.x * 256ll + threadIdx.x;
  if (e >= NN) return;
  const zd g = G[b * NN + e];
  G00[b * NN + e] = g;
  GT0[b * NN + e] = g;
  GTT[b * NN + e] = g;
  G0T[b * NN + e] = (e % N == e / N) ? zmk(g.x - 1.0, g.y) : g;
}

// X(i, j) = conj(Q(j, i)) / D(i)   (D^-1 Q^H of the QR of V1, for V1^-1 = P R^-1 D^-1 Q^H)
__global__ void k_scaled_adjoint(const zd* Q, const double* D, zd* X, int N) {
  const long long NN = (long long)N * N, b = blockIdx.y;
  const long long e = blockIdx.x * 256ll + threadIdx.x;
  if (e >= NN) return;
  const int i = e % N, j = e / N;
  const zd q = Q[b * NN + j + (long long)i * N];
  const double s = 1.0 / D[b * N + i];
  X[b * NN + e] = zmk(q.x * s, -q.y * s);
}

// out(jpvt_i - 1, :) = Y(i, :)   (row permutation P Y)
__global__ void k_perm_rows(const zd* Y, const int* jpvt, zd* out, int N) {
  const long long NN = (long long)N * N, b = blockIdx.y;
  const long long e = blockIdx.x * 256ll + threadIdx.x;
  if (e >= NN) return;
  const int i = e % N, j = e / N;
  out[b * NN + (jpvt[b * N + i] - 1) + (long long)j * N] = Y[b * NN + e];
}

// The 2N x 2N system of CGR2_2 (cgr2_2_mod.F90:338-378): first = D1(1) > D2(1);
//   HLPB2 = [[TL, TR], [BL, BR]], TL/BR = V1^-1 and U2^H (swapped unless first),
//   TR/BL = D1 U1^H and -D2 V2 (swapped unless first);  HLPB1 = HLPB2^H.
// grid (ceil(NN/256), B)
__global__ void k_cgr22_build(const zd* U1, const double* D1, const zd* V1I, const zd* U2, const double* D2,
                              const zd* V2, zd* HB2, zd* HB1, int* first, int N) {
  const long long NN = (long long)N * N, b = blockIdx.y;
  const long long e = blockIdx.x * 256ll + threadIdx.x;
  const int N2 = 2 * N;
  const long long NN2 = (long long)N2 * N2;
  const bool fst = D1[b * N] > D2[b * N];
  if (e == 0) first[b] = fst;
  if (e >= NN) return;
  const int i = e % N, j = e / N;
  const zd myu2 = zconj(U2[b * NN + j + (long long)i * N]);
  const zd v1i = V1I[b * NN + e];
  const zd u1h = zconj(U1[b * NN + j + (long long)i * N]);
  const zd a = zscale(u1h, D1[b * N + i]);
  const zd bb = zscale(V2[b * NN + e], -D2[b * N + i]);
  const zd tl = fst ? v1i : myu2, br = fst ? myu2 : v1i;
  const zd tr = fst ? a : bb, bl = fst ? bb : a;
  zd* H2 = HB2 + b * NN2;
  zd* H1 = HB1 + b * NN2;
  const int r[4] = {i, i, i + N, i + N}, c[4] = {j, j + N, j, j + N};
  const zd v[4] = {tl, tr, bl, br};
#pragma unroll
  for (int t = 0; t < 4; ++t) {
    H2[r[t] + (long long)c[t] * N2] = v[t];
    H1[c[t] + (long long)r[t] * N2] = zconj(v[t]);
  }
}

// HLP = rows of blockdiag(TL, BR) in pivot order (solve_extended_System's ZLAPMR
// forward, cgr2_2_mod.F90:172-176); TL / BR are read from HLPB2.  grid (ceil(4NN/256), B)
__global__ void k_cgr22_hlp(const zd* HB2, const int* jpvt, zd* HLP, int N) {
  const int N2 = 2 * N;
  const long long NN2 = (long long)N2 * N2, b = blockIdx.y;
  const long long e = blockIdx.x * 256ll + threadIdx.x;
  if (e >= NN2) return;
  const int i = e % N2, j = e / N2;
  const int r = jpvt[b * N2 + i] - 1;
  const bool in = (r < N && j < N) || (r >= N && j >= N);
  HLP[b * NN2 + e] = in ? HB2[b * NN2 + r + (long long)j * N2] : zmk(0.0, 0.0);
}

// X(i, :) *= 1 / D(i), D real (solve_extended_System: conj(1/D3) = 1/D3)
__global__ void k_scale_rows_inv(zd* X, const double* D, int N) {
  const long long NN = (long long)N * N, b = blockIdx.y;
  const long long e = blockIdx.x * 256ll + threadIdx.x;
  if (e >= NN) return;
  X[b * NN + e] = zscale(X[b * NN + e], 1.0 / D[b * N + e % N]);
}

// get_blocks (cgr2_2_mod.F90:55-73) of the solution into GRT0, GR00, GRTT, GR0T:
// first: (GR00, GR0T; GRT0, GRTT) = X, else (GRTT, GRT0; GR0T, GR00) = X.
__global__ void k_cgr22_blocks(const zd* X, const int* first, zd* GRT0, zd* GR00, zd* GRTT, zd* GR0T, int N) {
  const long long NN = (long long)N * N, b = blockIdx.y;
  const long long e = blockIdx.x * 256ll + threadIdx.x;
  if (e >= NN) return;
  const int N2 = 2 * N, i = e % N, j = e / N;
  const zd* x = X + b * (long long)N2 * N2;
  const zd A = x[i + (long long)j * N2], B = x[i + (long long)(j + N) * N2];
  const zd C = x[(i + N) + (long long)j * N2], D = x[(i + N) + (long long)(j + N) * N2];
  if (first[b]) {
    GR00[b * NN + e] = A; GR0T[b * NN + e] = B; GRT0[b * NN + e] = C; GRTT[b * NN + e] = D;
  } else {
    GRTT[b * NN + e] = A; GRT0[b * NN + e] = B; GR0T[b * NN + e] = C; GR00[b * NN + e] = D;
  }
}

// Control_Precision_tau for the four comparisons of one stabilisation: cmp[k][b] = {max |d|^2, mean |d|}
// (k_compare layout); stat slots 4..6 = ncg_tau, sum of means, max.  grid (ceil(C/128)), 128 threads
__global__ void k_tau_stats(const double* cmp, int C, int F, double* stat) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= C) return;
  double* st = stat + 8ll * c;
  for (int f = 0; f < F; ++f)
    for (int k = 0; k < 4; ++k) {
      const double* q = cmp + 2ll * (k * C * F + c * F + f);
      const double xmax = sqrt(q[0]);
      st[4] += 1.0;
      st[5] += q[1];
      if (xmax > st[6]) st[6] = xmax;
    }
}

// Quartet staging for ham%ObserT: out[chain][4][F][N][N] = [GT0, G0T, G00, GTT].
__global__ void k_gather_quartet(const zd* GT0, const zd* G0T, const zd* G00, const zd* GTT, zd* out, int N, int F) {
  const long long NN = (long long)N * N, b = blockIdx.y;
  const long long e = blockIdx.x * 256ll + threadIdx.x;
  if (e >= NN) return;
  const int c = b / F, f = b % F;
  zd* o = out + (long long)c * 4 * F * NN + (long long)f * NN + e;
  o[0] = GT0[b * NN + e];
  o[(long long)F * NN] = G0T[b * NN + e];
  o[2ll * F * NN] = G00[b * NN + e];
  o[3ll * F * NN] = GTT[b * NN + e];
}
