// Small per-slice and per-stabilisation kernels.
#pragma once
#include "common.cuh"
#include "linalg.cuh"

// Diagonal product of all single-site vertex exponentials of slice nt1 (1-based):
//   S(i) = prod_{n: P(n)=i} E_exp(1, s(n,nt1)),  Sinv(i) = prod E_exp(1, -s(n,nt1)).
// This is Op_mmultR / Op_Wrapup for diagonal operators (Operator_mod.F90:686-693,
// 776-781) for every vertex of the slice at once.  grid (B), block 256.
// sptr/slist: per (chain, flavour) the positions (vertex n, eigen-index I) of each site
// in ascending order, coded 2n + I (CSR, built at upload); Eexp: [k][I][s+2].
__global__ void k_slice_scale(const int8_t* fields, int L, int M, int N, int F, int nt1, const int* sptr,
                              const int* slist, const zd* Eexp, zd* S, zd* Sinv) {
  const int b = blockIdx.x, c = b / F, f = b % F;
  const int8_t* fl = fields + (long long)c * L * M + (long long)(nt1 - 1) * M;
  const int* ptr = sptr + (long long)b * (N + 1);
  const int* lst = slist + (long long)b * 2 * M;
  const zd* ee = Eexp + ((long long)c * F * M + (long long)f * M) * 10;
  for (int i = threadIdx.x; i < N; i += blockDim.x) {
    zd s = zmk(1.0, 0.0), si = zmk(1.0, 0.0);
    for (int e = ptr[i]; e < ptr[i + 1]; ++e) {
      const int code = lst[e], n = code >> 1, I = code & 1;
      const int sp = fl[n];
      s = zmul(s, ee[(long long)(2 * n + I) * 5 + sp + 2]);
      si = zmul(si, ee[(long long)(2 * n + I) * 5 - sp + 2]);
    }
    S[(long long)b * N + i] = s;
    Sinv[(long long)b * N + i] = si;
  }
}

// G(i,j) <- S(i) G(i,j) Sinv(j)  (deferred vertex wraps of one slice), grid (ceil(N*N/256), B)
__global__ void k_apply_scale(zd* G, const zd* S, const zd* Sinv, int N) {
  const int b = blockIdx.y;
  const long long NN = (long long)N * N;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < NN; e += (long long)gridDim.x * blockDim.x) {
    int i = e % N, j = e / N;
    zd* g = G + b * NN + e;
    *g = zmul(zmul(S[(long long)b * N + i], *g), Sinv[(long long)b * N + j]);
  }
}

// U = I, V = I, D = 1, det(U) = 1 (reset_UDV_state, udv_state_mod.F90:320-345)
__global__ void k_udv_reset(zd* U, zd* V, double* D, zd* detU, int N) {
  const int b = blockIdx.y;
  const long long NN = (long long)N * N;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < NN; e += (long long)gridDim.x * blockDim.x) {
    int i = e % N, j = e / N;
    zd v = zmk(i == j ? 1.0 : 0.0, 0.0);
    U[b * NN + e] = v;
    V[b * NN + e] = v;
    if (e < N) D[(long long)b * N + e] = 1.0;
    if (e == 0) detU[b] = zmk(1.0, 0.0);
  }
}

// decompose_UDV_state phase handling (udv_state_mod.F90:481-492): phase = prod R_ii *
// pivot sign (conjugated on the L side); R(1,:) /= phase; det(U) = det(Q) * phase.
__global__ void k_decomp_phase(zd* R, long long ldr, int N, const QRInfo* info, int left, zd* phase_out, zd* detU) {
  const int b = blockIdx.x;
  __shared__ zd s_beta;
  if (threadIdx.x == 0) {
    zd ph = info[b].prodR;
    if (info[b].psign < 0) ph = zneg(ph);
    if (left) ph = zconj(ph);
    phase_out[b] = ph;
    detU[b] = zmul(info[b].detQ, ph);
    s_beta = zdiv(zmk(1.0, 0.0), ph);
  }
  __syncthreads();
  zd* Rb = R + (long long)b * ldr * N;
  for (int j = threadIdx.x; j < N; j += blockDim.x) Rb[(long long)j * ldr] = zmul(s_beta, Rb[(long long)j * ldr]);
}

// U(:,1) *= phase
__global__ void k_scale_col0(zd* U, int N, const zd* phase) {
  const int b = blockIdx.x;
  zd* u = U + (long long)b * N * N;
  zd ph = phase[b];
  for (int r = threadIdx.x; r < N; r += blockDim.x) u[r] = zmul(u[r], ph);
}

// COMPARE_C (mymats_mod.F90:683-704) with the NaN test of Control_PrecisionG
// (control_mod.F90:219-263).  grid (CMP_BLOCKS, B), block 256; out[b] = {xmax, xmean},
// zeroed by the caller.  The maximum is taken over |d|^2 as an integer on the IEEE bit
// pattern (non-negative doubles order like their bits) and rooted once; the mean adds
// FP32 square roots per element (a diagnostic) in FP64 partial sums.  Per element this
// costs five FP64-pipe instructions instead of a hypot.
#define CMP_BLOCKS 32
__global__ void __launch_bounds__(256) k_compare(const zd* A, const zd* Bm, int N, double* out, int* err) {
  const int b = blockIdx.y;
  const long long NN = (long long)N * N;
  const zd* a = A + b * NN;
  const zd* c = Bm + b * NN;
  unsigned long long mx = 0ull;
  float sm = 0.f;
  int nan = 0;
  for (long long e = blockIdx.x * 256ll + threadIdx.x; e < NN; e += 256ll * CMP_BLOCKS) {
    const zd x = a[e], y = c[e];
    const unsigned long long bits[4] = {(unsigned long long)__double_as_longlong(x.x),
                                        (unsigned long long)__double_as_longlong(x.y),
                                        (unsigned long long)__double_as_longlong(y.x),
                                        (unsigned long long)__double_as_longlong(y.y)};
#pragma unroll
    for (int t = 0; t < 4; ++t) nan |= (bits[t] & 0x7fffffffffffffffull) > 0x7ff0000000000000ull;
    const double dx = x.x - y.x, dy = x.y - y.y;
    const double d2 = fma(dx, dx, dy * dy);
    const unsigned long long u = (unsigned long long)__double_as_longlong(d2);
    mx = u > mx ? u : mx;
    sm += sqrtf(__double2float_rn(d2));
  }
  __shared__ unsigned long long rm[8];
  __shared__ float rs[8];
  __shared__ int rn[8];
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long om = __shfl_xor_sync(0xffffffffu, mx, o);
    mx = om > mx ? om : mx;
    sm += __shfl_xor_sync(0xffffffffu, sm, o);
  }
  nan = __any_sync(0xffffffffu, nan);
  if ((threadIdx.x & 31) == 0) { rm[threadIdx.x >> 5] = mx; rs[threadIdx.x >> 5] = sm; rn[threadIdx.x >> 5] = nan; }
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned long long m = 0ull;
    double s = 0.0;
    int nn = 0;
    for (int w = 0; w < 8; ++w) { m = rm[w] > m ? rm[w] : m; s += (double)rs[w]; nn |= rn[w]; }
    if (m > 0x7ff0000000000000ull) nn = 1;
    atomicMax(reinterpret_cast<unsigned long long*>(out + 2 * b), m);  // |d|^2 bits; rooted by k_stab_finish
    atomicAdd(out + 2 * b + 1, s / (double)NN);
    if (nn) atomicOr(err, 1);
  }
}

// Op_phase angle sum (Operator_mod.F90:160-181): sum over n, nt of Im(g alpha phi).
__global__ void k_opphase(const int8_t* fields, int L, int M, int F, const zd* g, const zd* alpha, const int8_t* type,
                          FieldTables ft, double* out) {
  const int b = blockIdx.x, c = b / F, f = b % F;
  const int8_t* fl = fields + (long long)c * L * M;
  const long long k0 = (long long)c * F * M + (long long)f * M;
  double s = 0.0;
  for (long long e = threadIdx.x; e < (long long)L * M; e += blockDim.x) {
    int n = e % M;
    int sp = fl[e];
    zd ga = zmul(g[k0 + n], alpha[k0 + n]);
    s += ga.y * ft.phi[type[(long long)c * F * M + n] - 1][sp + 2];
  }
  __shared__ double r[8];
  s = warp_sum(s);
  if ((threadIdx.x & 31) == 0) r[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += r[w];
    out[b] = t;
  }
}

// Phase and precision bookkeeping after CGR on all flavours of a chain
// (main.F90:734-753, control_mod.F90:207-320).  stat layout per chain:
// [0] ncg [1] xmeanG_sum [2] xmaxG [3] xmaxP [4] ncg_tau [5] xmean_tau_sum [6] xmax_tau [7] sweeps
struct StabFinishParams {
  int C, F, NSUN, nvar, compare, init;
  const zd* detUR; const zd* detUL;   // [B]
  const QRInfo* info;                 // [B]
  const double* opang;                // [B]
  const double* cmp;                  // [B][2]
  zd* phase;                          // [C]
  double* stat;                       // [C][8]
  int* err;
  zd* rec_phase;                      // [C] slot for this point or null
};

__global__ void k_stab_finish(StabFinishParams p) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= p.C) return;
  zd Z = zmk(1.0, 0.0);
  double* st = p.stat + 8ll * c;
  for (int f = 0; f < p.F; ++f) {
    const int b = c * p.F + f;
    zd ph = zmul(p.detUR[b], zconj(p.detUL[b]));  // conj(det(U_R^H U_L))
    ph = zscale(ph, 1.0 / zabs(ph));
    if (p.info[b].psign < 0) ph = zneg(ph);
    zd q = zmul(p.info[b].prodR, p.info[b].detQ);
    if (p.nvar != 1) q = zconj(q);
    ph = zmul(ph, q);
    double s, co;
    sincos(p.opang[b], &s, &co);
    ph = zmul(ph, zmk(co, s));
    Z = zmul(Z, ph);
    if (p.compare) {
      double xmax = sqrt(p.cmp[2 * b]), xmean = p.cmp[2 * b + 1];  // k_compare leaves max |d|^2
      st[0] += 1.0;
      if (xmax > 10.0) atomicOr(p.err, 2);
      if (xmax > st[2]) st[2] = xmax;
      st[1] += xmean;
    }
  }
  zd Zp = Z;
  for (int e = 1; e < p.NSUN; ++e) Zp = zmul(Zp, Z);
  if (p.compare) {
    double X = zabs(zsub(Zp, p.phase[c]));
    if (X > st[3]) st[3] = X;
  }
  p.phase[c] = Zp;
  if (p.rec_phase) p.rec_phase[c] = Zp;
}

__global__ void k_real_to_complex(const double* a, zd* out, long long n) {
  long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i < n) out[i] = zmk(a[i], 0.0);
}
__global__ void k_real_to_complex2(const double* a, const double* b, zd* oa, zd* ob, long long n) {
  long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i < n) {
    oa[i] = zmk(a[i], 0.0);
    ob[i] = zmk(b[i], 0.0);
  }
}
// per-batch flush rank: out[c*F + f] = m[c]
__global__ void k_expand_m(const int* m, int* out, int C, int F) {
  int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b < C * F) out[b] = m[b / F];
}
__global__ void k_count_sweep(double* stat, int C) {
  int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c < C) stat[8 * c + 7] += 1.0;
}

// G <- W G W^T for the block-diagonal real orthogonal W with the 2x2 block U (column-major)
// on every site pair: the rotated-basis G of two-site vertices back to the original basis.
// Rows: grid (ceil(N*npairs/256), B); columns: the same grid.
__global__ void k_rot_rows(zd* G, int N, const int* pairs, int npairs, double u00, double u10, double u01,
                           double u11) {
  const long long NN = (long long)N * N, b = blockIdx.y;
  const long long e = blockIdx.x * 256ll + threadIdx.x;
  if (e >= (long long)N * npairs) return;
  const int j = e % N, pr = e / N;
  zd* g = G + b * NN + (long long)j * N;
  const int a = pairs[2 * pr], c = pairs[2 * pr + 1];
  const zd x = g[a], y = g[c];
  g[a] = zadd(zscale(x, u00), zscale(y, u01));
  g[c] = zadd(zscale(x, u10), zscale(y, u11));
}
__global__ void k_rot_cols(zd* G, int N, const int* pairs, int npairs, double u00, double u10, double u01,
                           double u11) {
  const long long NN = (long long)N * N, b = blockIdx.y;
  const long long e = blockIdx.x * 256ll + threadIdx.x;
  if (e >= (long long)N * npairs) return;
  const int i = e % N, pr = e / N;
  zd* g = G + b * NN;
  const int a = pairs[2 * pr], c = pairs[2 * pr + 1];
  const zd x = g[i + (long long)a * N], y = g[i + (long long)c * N];
  g[i + (long long)a * N] = zadd(zscale(x, u00), zscale(y, u01));
  g[i + (long long)c * N] = zadd(zscale(x, u10), zscale(y, u11));
}


// Equal-time scalar observables of the Hubbard-type models at one ham%Obser call site
// (Hamiltonian_Hubbard_smod.F90:695-801; kinetic term as Predefined_Hoppings_Compute_Kin,
// Predefined_Hop_mod.F90:1905-1959), accumulated per chain:
//   GRC(i,j) = delta_ij - G(j,i),  ZP = Phase / Re(Phase),  ZS = sign(Re(Phase))
//   Kin  = N_SUN sum_f sum_ij H_f(i,j) GRC_f(i,j) = N_SUN sum_f [tr H_f - sum_ij H_f(i,j) G_f(j,i)]
//   Pot  = sum_i U_i GRC_1(i,i) GRC_dec(i,i)   (dec = 2 for two flavours, else 1)
//   Part = N_SUN sum_f sum_i GRC_f(i,i),  Ener = Kin + Pot
// acc[c] += {ZP ZS Kin, ZP ZS Pot, ZP ZS Part, ZP ZS Ener} (complex), ZS, 1.
// HT holds H_f transposed (HT_f[j + i N] = H_f(i,j)), so sum_ij H(i,j) G(j,i) is the
// elementwise sum over the two column-major arrays.  One CTA (256 threads) per chain, fixed
// summation order.
__global__ void __launch_bounds__(256) k_obs_scal(const zd* G, const zd* phase, const double* HT, const double* trH,
                                                  const double* U, int N, int F, int nsun, double* acc) {
  const int c = blockIdx.x, tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const long long NN = (long long)N * N;
  double kr = 0.0, ki = 0.0, pr = 0.0, pi = 0.0;
  for (int f = 0; f < F; ++f) {
    const zd* g = G + ((long long)c * F + f) * NN;
    const double* ht = HT + (long long)f * NN;
    for (long long e = tid; e < NN; e += 256) {
      const zd v = g[e];
      kr = fma(ht[e], v.x, kr);
      ki = fma(ht[e], v.y, ki);
    }
  }
  // Pot and Part need the diagonals of both flavours at the same site
  double rr = 0.0, ri = 0.0;
  for (int i = tid; i < N; i += 256) {
    const zd g1 = G[((long long)c * F) * NN + i + (long long)i * N];
    const zd a = zmk(1.0 - g1.x, -g1.y);  // GRC_1(i,i)
    zd b = a;
    if (F == 2) {
      const zd g2 = G[((long long)c * F + 1) * NN + i + (long long)i * N];
      b = zmk(1.0 - g2.x, -g2.y);
      rr += b.x; ri += b.y;
    }
    rr += a.x; ri += a.y;
    const zd ab = zmul(a, b);
    pr = fma(U[i], ab.x, pr);
    pi = fma(U[i], ab.y, pi);
  }
  double v[6] = {kr, ki, pr, pi, rr, ri};
#pragma unroll
  for (int q = 0; q < 6; ++q) v[q] = warp_sum(v[q]);
  __shared__ double wsum[6][8];
  if (lane == 0)
    for (int q = 0; q < 6; ++q) wsum[q][warp] = v[q];
  __syncthreads();
  if (tid == 0) {
    double s[6];
    for (int q = 0; q < 6; ++q) {
      s[q] = 0.0;
      for (int w = 0; w < 8; ++w) s[q] += wsum[q][w];
    }
    double trh = 0.0;
    for (int f = 0; f < F; ++f) trh += trH[f];
    const zd kin = zmk(nsun * (trh - s[0]), -nsun * s[1]);
    const zd pot = zmk(s[2], s[3]);
    const zd part = zmk(nsun * s[4], nsun * s[5]);  // s[4], s[5]: sum_f sum_i GRC_f(i,i)
    const zd ph = phase[c];
    const double zs = ph.x > 0.0 ? 1.0 : (ph.x < 0.0 ? -1.0 : 0.0);
    const zd zpzs = ph.x != 0.0 ? zscale(zmk(1.0, ph.y / ph.x), zs) : zmk(0.0, 0.0);
    const zd o[4] = {kin, pot, part, zadd(kin, pot)};
    double* a = acc + 10ll * c;
    for (int q = 0; q < 4; ++q) {
      const zd w = zmul(o[q], zpzs);
      a[2 * q] += w.x;
      a[2 * q + 1] += w.y;
    }
    a[8] += zs;
    a[9] += 1.0;
  }
}

// ---- explicit vertex wraps of one phase (models with vector vertices) --------------------------
// A phase is a range [n0, n1) of vertices with pairwise disjoint supports in the rotated basis.
// Vertex n acts on its support with the block
//   kind 0 (one site a):            e_0
//   kind 1 (pair (a, b), diagonal): diag(e_0, e_1)
//   kind 2 (pair (a, b), vector u): I + (e_0 - 1) u u^T,  u = (c_a, c_b) real, |u| = 1
// where e_m = E_exp(m, s) of the vertex's field s (Op%E_exp of Operator_mod.F90:472-529), with
// s -> -s for the inverse (inv) and every entry conjugated for the adjoint (cj; the blocks
// are symmetric).  fl points at the slice's fields of chain 0 ([chain] stride fstride).
struct VtxPhase {
  const int8_t* fl; long long fstride;
  const int8_t* kind; const int* site; const int* site2; const double* coef;  // [chain][F*M]
  const zd* Eexp;                                                              // [chain][F*M][2][5]
  long long sK;                                                                // F * M
  int F, M, N, n0, n1, inv, cj;
};

ALF_DEV void vtx_block(const VtxPhase& p, int b, int n, int* a, int* c, zd m[4], int* two) {
  const int ch = b / p.F, f = b % p.F;
  const long long k = (long long)ch * p.sK + (long long)f * p.M + n;
  int s = p.fl[(long long)ch * p.fstride + n];
  if (p.inv) s = -s;
  const zd* ee = p.Eexp + k * 10;
  const zd e0 = ee[s + 2];
  const int kd = p.kind[k];
  *a = p.site[k];
  *two = kd != 0;
  if (kd == 0) {
    m[0] = e0;
  } else if (kd == 1) {
    *c = p.site2[k];
    m[0] = e0; m[1] = zmk(0.0, 0.0); m[2] = zmk(0.0, 0.0); m[3] = ee[5 + s + 2];
  } else {
    *c = p.site2[k];
    const double ua = p.coef[2 * k], ub = p.coef[2 * k + 1];
    const zd d = zmk(e0.x - 1.0, e0.y);
    m[0] = zadd(zmk(1.0, 0.0), zscale(d, ua * ua));
    m[1] = zscale(d, ua * ub);  // (b, a) entry
    m[2] = m[1];                 // (a, b) entry
    m[3] = zadd(zmk(1.0, 0.0), zscale(d, ub * ub));
  }
  if (p.cj)
    for (int e = 0; e < 4; ++e) m[e] = zconj(m[e]);
}

// X <- E X (rows of every vertex's support), grid (ceil(N * (n1 - n0) / 256), B)
__global__ void k_vtx_rows(zd* X, long long sX, VtxPhase p) {
  const int b = blockIdx.y;
  const long long e = blockIdx.x * 256ll + threadIdx.x;
  const int nv = p.n1 - p.n0;
  if (e >= (long long)p.N * nv) return;
  const int j = (int)(e % p.N), n = p.n0 + (int)(e / p.N);
  int a = 0, c = 0, two = 0;
  zd m[4];
  vtx_block(p, b, n, &a, &c, m, &two);
  zd* col = X + b * sX + (long long)j * p.N;
  if (!two) { col[a] = zmul(m[0], col[a]); return; }
  const zd xa = col[a], xc = col[c];
  col[a] = zadd(zmul(m[0], xa), zmul(m[2], xc));
  col[c] = zadd(zmul(m[1], xa), zmul(m[3], xc));
}

// X <- X E (columns of every vertex's support), grid (ceil(N * (n1 - n0) / 256), B)
__global__ void k_vtx_cols(zd* X, long long sX, VtxPhase p) {
  const int b = blockIdx.y;
  const long long e = blockIdx.x * 256ll + threadIdx.x;
  const int nv = p.n1 - p.n0;
  if (e >= (long long)p.N * nv) return;
  const int i = (int)(e % p.N), n = p.n0 + (int)(e / p.N);
  int a = 0, c = 0, two = 0;
  zd m[4];
  vtx_block(p, b, n, &a, &c, m, &two);
  zd* Xb = X + b * sX;
  if (!two) { Xb[i + (long long)a * p.N] = zmul(Xb[i + (long long)a * p.N], m[0]); return; }
  const zd xa = Xb[i + (long long)a * p.N], xc = Xb[i + (long long)c * p.N];
  Xb[i + (long long)a * p.N] = zadd(zmul(xa, m[0]), zmul(xc, m[1]));
  Xb[i + (long long)c * p.N] = zadd(zmul(xa, m[2]), zmul(xc, m[3]));
}

// copy of one slice's fields of every chain (the fields before the slice's updates)
__global__ void k_copy_fields(const int8_t* fields, int L, int M, int nt1, int8_t* out) {
  const int c = blockIdx.y;
  for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < M; n += gridDim.x * blockDim.x)
    out[(long long)c * M + n] = fields[(long long)c * L * M + (long long)(nt1 - 1) * M + n];
}

// ---- checkerboard hopping: bond operators of one family ------------------------------------
// Bonds [b0, b1) of a family are disjoint two-site operators (P [F][ncheck][2], E [F][ncheck][4]
// real, column-major 2 x 2); batch entry b uses flavour b % F.  The RealExpOpT lmult / rmult of
// each bond (Prog/OpTTypes_mod.F90:135-304): rows (X <- E X) or columns (X <- X E).
// grid (ceil(N (b1 - b0) / 256), B)
__global__ void k_bond_rows(zd* X, long long sX, int N, int F, const int* P, const double* E, int ncheck, int b0,
                            int b1) {
  const int b = blockIdx.y, f = b % F;
  const long long e = blockIdx.x * 256ll + threadIdx.x;
  if (e >= (long long)N * (b1 - b0)) return;
  const int j = (int)(e % N), nc = b0 + (int)(e / N);
  const long long k = (long long)f * ncheck + nc;
  const int a = P[2 * k], c = P[2 * k + 1];
  const double* m = E + 4 * k;
  zd* col = X + b * sX + (long long)j * N;
  const zd xa = col[a], xc = col[c];
  col[a] = zadd(zscale(xa, m[0]), zscale(xc, m[2]));
  col[c] = zadd(zscale(xa, m[1]), zscale(xc, m[3]));
}
__global__ void k_bond_cols(zd* X, long long sX, int N, int F, const int* P, const double* E, int ncheck, int b0,
                            int b1) {
  const int b = blockIdx.y, f = b % F;
  const long long e = blockIdx.x * 256ll + threadIdx.x;
  if (e >= (long long)N * (b1 - b0)) return;
  const int i = (int)(e % N), nc = b0 + (int)(e / N);
  const long long k = (long long)f * ncheck + nc;
  const int a = P[2 * k], c = P[2 * k + 1];
  const double* m = E + 4 * k;
  zd* Xb = X + b * sX;
  const zd xa = Xb[i + (long long)a * N], xc = Xb[i + (long long)c * N];
  Xb[i + (long long)a * N] = zadd(zscale(xa, m[0]), zscale(xc, m[1]));
  Xb[i + (long long)c * N] = zadd(zscale(xa, m[2]), zscale(xc, m[3]));
}

// X(i, j) *= rs(i) (conjugated with rconj) * cs(j); rs or cs may be null.  grid (ceil(N N / 256), B)
__global__ void k_scale_rc(zd* X, int N, const zd* rs, int rconj, const zd* cs) {
  const int b = blockIdx.y;
  const long long NN = (long long)N * N;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < NN; e += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(e % N), j = (int)(e / N);
    zd v = X[b * NN + e];
    if (rs) v = zmul(rconj ? zconj(rs[(long long)b * N + i]) : rs[(long long)b * N + i], v);
    if (cs) v = zmul(v, cs[(long long)b * N + j]);
    X[b * NN + e] = v;
  }
}
