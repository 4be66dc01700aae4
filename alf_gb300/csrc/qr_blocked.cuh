// Blocked Householder QR with norm pre-pivoting, and the explicit Q.
//
// Pivoting follows ALF's STABLOG branch of decompose_UDV_state
// (Prog/udv_state_mod.F90:503-542): the columns are ordered once by their
// norms (log|A(:,j)| + log(scale_j)), then factored without pivoting
// (QDRP_decompose with IPVT = 1).  Each Householder step is ZLARFG (beta,
// tau, 1/(alpha-beta)) and the left application of H^H = I - conj(tau) v v^H
// (LAPACK ZGEQR2 as vendored in Libraries/libqrref), followed by QDRP's
// D = |R_ii| and row normalisation (Prog/QDRP_decompose_mod.F90:85-100).
//
// GB300 layout of the work: FP64 DMMA and DFMA run at the same ~1 TFLOP/s,
// so a GEMM-shaped trailing update buys nothing over applying the panel's
// reflectors column by column; what matters is that the trailing work is
// spread over all SMs and that the sequential chain per column is short.
//   k_bqr_keys     column keys (one warp per column, all SMs)
//   k_bqr_permute  rank sort of the keys, permuted + scaled copy, jpvt, sign
//   k_bqr_panel    one panel of nb <= 32 columns on a thread-block cluster:
//                  rows dealt in contiguous chunks to the CTAs, ONE
//                  distributed-shared-memory exchange per column carries the
//                  norm, all dot products v^H a_j of the panel and the pivot row
//   k_bqr_apply    the panel's reflectors applied to every later column, one
//                  warp per column, all SMs (also used for Q, in reverse)
//   k_bqr_finish   D, row normalisation, det(Q) and prod R_ii/|R_ii|
#pragma once
#include "common.cuh"
#include "linalg.cuh"
#include "arith.cuh"

#define BQR_NB 32
#define BQR_ROWS 32   // max rows of a panel per CTA (N <= 32 * cluster size)
#define BQR_LROWS 24  // max rows per lane in k_bqr_apply (N <= 768)

// 1/d for real d != 0: float seed and two Newton-Raphson steps (an FP64 division
// costs ~560 dependent cycles on GB300); falls back to division outside float range.
ALF_DEV double bqr_rcp(double d) {
  const double a = fabs(d);
  if (!(a > 1e-30 && a < 1e30)) return 1.0 / d;
  double r = (double)__frcp_rn(__double2float_rn(d));
  r = fma(r, fma(-d, r, 1.0), r);
  return fma(r, fma(-d, r, 1.0), r);
}
ALF_DEV zd bqr_zrcp(zd a) {
  const double s = bqr_rcp(a.x * a.x + a.y * a.y);
  return zmk(a.x * s, -a.y * s);
}

// keys[b][j] = log ||A(:,j)|| + log |scale_j|  (-inf for a zero column)
__global__ void __launch_bounds__(256) k_bqr_keys(const zd* A, long long lda, long long sA, int N,
                                                  const double* scale, long long sS, double* keys) {
  const int b = blockIdx.y, lane = threadIdx.x & 31;
  const int c = blockIdx.x * 8 + (threadIdx.x >> 5);
  if (c >= N) return;
  const zd* col = A + b * sA + (long long)c * lda;
  double s = 0.0;
  for (int r = lane; r < N; r += 32) s = fma(col[r].x, col[r].x, fma(col[r].y, col[r].y, s));
  s = warp_sum(s);
  if (lane == 0) {
    double k = (s > 0.0) ? 0.5 * log(s) : -INFINITY;
    if (scale) k += log(fabs(scale[b * sS + c]));
    keys[(long long)b * N + c] = k;
  }
}

// Rank sort (descending key, ties by index), Out(:, i) = A(:, jpvt_i - 1) * scale,
// jpvt 1-based like LAPACK; block x == 0 also writes jpvt and the permutation sign.
// grid (ceil(N/8), B), 256 threads; dynamic smem: N doubles + N ints.
__global__ void __launch_bounds__(256) k_bqr_permute(const zd* A, long long lda, long long sA, int N,
                                                     const double* scale, long long sS, const double* keys,
                                                     zd* Out, long long sO, int* jpvt, long long sP, QRInfo* info) {
  const int b = blockIdx.y, tid = threadIdx.x;
  extern __shared__ double kbuf[];
  int* src = reinterpret_cast<int*>(kbuf + N);  // src[rank] = original column
  __shared__ int inv_cnt;
  for (int j = tid; j < N; j += 256) {
    double v = keys[(long long)b * N + j];
    kbuf[j] = (v != v) ? -INFINITY : v;  // NaN keys sort last
  }
  if (tid == 0) inv_cnt = 0;
  __syncthreads();
  for (int j = tid; j < N; j += 256) {
    const double kj = kbuf[j];
    int r = 0;
    for (int i = 0; i < N; ++i) {
      const double ki = kbuf[i];
      r += (ki > kj) || (ki == kj && i < j);
    }
    src[r] = j;
  }
  __syncthreads();
  if (blockIdx.x == 0) {
    int cnt = 0;  // inversions of src, for the sign
    for (int j = tid; j < N; j += 256) {
      const int sj = src[j];
      for (int i = 0; i < j; ++i) cnt += src[i] > sj;
      jpvt[b * sP + j] = sj + 1;
    }
    atomicAdd(&inv_cnt, cnt & 1);
    __syncthreads();
    if (tid == 0) info[b].psign = (inv_cnt & 1) ? -1 : 1;
  }
  const int lane = tid & 31;
  const int i = blockIdx.x * 8 + (tid >> 5);
  if (i >= N) return;
  const int s = src[i];
  const double sc = scale ? scale[b * sS + s] : 1.0;
  const zd* in = A + b * sA + (long long)s * lda;
  zd* out = Out + b * sO + (long long)i * lda;
  for (int r = lane; r < N; r += 32) out[r] = scale ? zscale(in[r], sc) : in[r];
}

struct BQRPanel {
  zd* A; long long lda, sA;  // factored in place
  int N, j0, nb;
  zd* tau; long long sT;
  double* D; long long sD;   // |R(kc,kc)| of the panel's columns
};

// One panel, columns [j0, j0+nb), rows [j0, N), on a cluster of CL CTAs of 256 threads.
// Thread (j = tid % 32, g = tid / 32) handles panel column j on the CTA's rows g, g+8, ...
__global__ void __launch_bounds__(256) k_bqr_panel(BQRPanel p) {
  const unsigned rank = cluster_ctarank(), CL = cluster_nctarank();
  const int b = blockIdx.y, N = p.N, j0 = p.j0, nb = p.nb;
  const int tid = threadIdx.x, j = tid & 31, g = tid >> 5;
  const int mp = N - j0;
  const int rpc = (mp + (int)CL - 1) / (int)CL;
  const int r0 = j0 + (int)rank * rpc;
  const int nr = max(0, min(N, r0 + rpc) - r0);
  zd* A = p.A + b * p.sA;
  const long long lda = p.lda;
  __shared__ zd P[BQR_ROWS][BQR_NB + 1];
  __shared__ zd red[8][BQR_NB];
  __shared__ zd xs[2][BQR_NB];  // this CTA's column partial sums (read remotely)
  __shared__ zd xr[2][BQR_NB];  // the pivot row, published by its owner
  __shared__ zd tot[BQR_NB], prow[BQR_NB];
  __shared__ double s_beta;
  __shared__ zd s_t, s_scal, s_alpha;
  __shared__ bool s_triv;
  for (int il = g; il < nr; il += 8)
    if (j < nb) P[il][j] = A[(r0 + il) + (long long)(j0 + j) * lda];
  __syncthreads();

  for (int k = 0; k < nb; ++k) {
    const int kc = j0 + k, par = k & 1;
    const unsigned owner = (unsigned)(k / rpc);
    // partials over own rows i > kc: column k -> sum |a_ik|^2, column j > k -> sum conj(a_ik) a_ij
    zd acc = zmk(0.0, 0.0);
    if (j >= k && j < nb)
      for (int il = g; il < nr; il += 8)
        if (r0 + il > kc) acc = zfma(zconj(P[il][k]), P[il][j], acc);
    red[g][j] = acc;
    if (rank == owner && j < nb && g == 0) xr[par][j] = P[kc - r0][j];
    __syncthreads();
    if (g == 0) {
      const zd s = zadd(zadd(zadd(red[0][j], red[1][j]), zadd(red[2][j], red[3][j])),
                        zadd(zadd(red[4][j], red[5][j]), zadd(red[6][j], red[7][j])));
      xs[par][j] = s;
    }
    cluster_sync();
    if (g == 0 && j >= k && j < nb) {
      zd s0 = zmk(0.0, 0.0), s1 = s0, s2 = s0, s3 = s0;
      for (unsigned q = 0; q < CL; q += 4) {
        const unsigned a0 = dsmem_addr(&xs[par][j], q);
        s0 = zadd(s0, zmk(dsmem_ld_f64(a0), dsmem_ld_f64(a0 + 8)));
        if (q + 1 < CL) { const unsigned a = dsmem_addr(&xs[par][j], q + 1); s1 = zadd(s1, zmk(dsmem_ld_f64(a), dsmem_ld_f64(a + 8))); }
        if (q + 2 < CL) { const unsigned a = dsmem_addr(&xs[par][j], q + 2); s2 = zadd(s2, zmk(dsmem_ld_f64(a), dsmem_ld_f64(a + 8))); }
        if (q + 3 < CL) { const unsigned a = dsmem_addr(&xs[par][j], q + 3); s3 = zadd(s3, zmk(dsmem_ld_f64(a), dsmem_ld_f64(a + 8))); }
      }
      tot[j] = zadd(zadd(s0, s1), zadd(s2, s3));
      const unsigned ar = dsmem_addr(&xr[par][j], owner);
      prow[j] = zmk(dsmem_ld_f64(ar), dsmem_ld_f64(ar + 8));
    }
    // ZLARFG on (alpha, x), x = A(kc+1:N, kc), by warp 0 only (every FP64 instruction costs
    // its sub-partition ~76 cycles; eight redundant copies would cost eight times that)
    if (g == 0) {
      __syncwarp();  // tot / prow were written by other lanes of this warp
      const zd alpha = prow[k];
      const double xn2 = tot[k].x;
      const bool triv = (xn2 == 0.0 && alpha.y == 0.0);
      double be = alpha.x;
      zd tt = zmk(0.0, 0.0), sc = zmk(0.0, 0.0);
      if (!triv) {
        be = -copysign(sqrt(fma(alpha.x, alpha.x, fma(alpha.y, alpha.y, xn2))), alpha.x);
        const double ib = bqr_rcp(be);
        tt = zmk((be - alpha.x) * ib, -alpha.y * ib);
        sc = bqr_zrcp(zmk(alpha.x - be, alpha.y));
      }
      if (j == 0) { s_beta = be; s_t = tt; s_scal = sc; s_triv = triv; s_alpha = alpha; }
    }
    __syncthreads();
    const bool trivial = s_triv;
    const double beta = s_beta;
    const zd t = s_t, scal = s_scal, alpha = s_alpha;
    // H^H applied to the panel's later columns: a_j -= conj(tau) v (v^H a_j),
    // v^H a_j = a_kc,j + conj(scal) sum_{i>kc} conj(a_ik) a_ij
    // v_i = scal a_ik for the warp's rows, read before any lane overwrites column k
    zd vi[BQR_ROWS / 8];
#pragma unroll
    for (int q = 0; q < BQR_ROWS / 8; ++q) {
      const int il = g + 8 * q;
      if (il >= nr) break;  // warp-uniform (il depends on the warp only)
      vi[q] = zmul(scal, P[il][k]);
    }
    __syncwarp();
    if (!trivial && j >= k && j < nb) {
      const zd f = (j > k) ? zmul(zconj(t), zadd(prow[j], zmul(zconj(scal), tot[j]))) : zmk(0.0, 0.0);
#pragma unroll
      for (int q = 0; q < BQR_ROWS / 8; ++q) {
        const int il = g + 8 * q;
        if (il >= nr) break;
        const int i = r0 + il;
        if (i > kc) {
          if (j == k) P[il][k] = vi[q];
          else P[il][j] = zfms(vi[q], f, P[il][j]);
        } else if (i == kc) {
          if (j == k) P[il][k] = zmk(beta, 0.0);
          else P[il][j] = zsub(P[il][j], f);
        }
      }
    }
    if (rank == owner && tid == 0) {
      p.tau[b * p.sT + kc] = t;
      p.D[b * p.sD + kc] = trivial ? zabs(alpha) : fabs(beta);
    }
    __syncthreads();
  }
  for (int il = g; il < nr; il += 8)
    if (j < nb) A[(r0 + il) + (long long)(j0 + j) * lda] = P[il][j];
  cluster_sync();  // no CTA leaves while its shared memory may still be read
}

struct BQRApply {
  const void* V; long long ldv, sV;  // reflectors (column kc holds v below row kc, v_kc = 1 implicit),
                                     // stored in the kernel's arithmetic (FP64 or double-float)
  const zd* tau; long long sT;
  zd* C; long long ldc, sC;          // columns c0 .. N-1 are updated, rows j0 .. N-1 (FP64)
  int N, j0, nb, c0;
  int conj_tau;  // 1: QR trailing update, H^H in order k = 0..nb-1
                 // 0: Q applied (ZUNMQR 'L','N'), H in reverse order
  int init;      // with conj_tau = 0: columns [j0, j0+nb) start as e_c (explicit Q, ZUNGQR)
};

// One column per CTA of 4 warps (one per SMSP: on GB300 a warp issues at most one
// FP64 instruction every ~64 cycles); grid (N - c0, B), 128 threads.  Warp w holds the
// 32-row blocks w, w+4, ... of rows j0..N-1 (lane l: row j0 + l + 32 (w + 4 q)); row
// blocks above the reflector are skipped warp-uniformly; the four warp partials of
// v^H x meet in shared memory (double-buffered: one barrier per reflector); the next
// reflector is prefetched.  Arithmetic A: ArD or ArF.
// WPC warps per column (4: latency, one per sub-partition; 1: throughput, when the
// columns of the launch already fill the GPU), QW 32-row blocks per warp (WPC * 32 * QW
// rows at most); launched with the smallest QW that covers the matrix (bqr_apply below).
template <class A, int QW, int WPC>
__global__ void __launch_bounds__(32 * WPC) k_bqr_apply(BQRApply p) {
  constexpr int BQR_QW = QW;
  typedef typename A::Z Z;
  const int b = blockIdx.y, lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int c = p.c0 + blockIdx.x;
  if (c >= p.N) return;
  const int N = p.N, j0 = p.j0, nb = p.nb;
  const int nblk = (N - j0 + 31) >> 5;  // 32-row blocks
  const Z* V = reinterpret_cast<const Z*>(p.V) + b * p.sV;
  constexpr int NWc = WPC;
  const zd* tau = p.tau + b * p.sT;
  zd* col = p.C + b * p.sC + (long long)c * p.ldc;
  const bool fresh = p.init && c < j0 + nb;
  __shared__ Z red[2][4];
  Z x[BQR_QW], vn[BQR_QW];
#pragma unroll
  for (int q = 0; q < BQR_QW; ++q) {
    const int blk = w + NWc * q, r = j0 + lane + 32 * blk;
    x[q] = A::zero();
    vn[q] = A::zero();
    if (blk < nblk && r < N) x[q] = fresh ? (r == c ? A::one() : A::zero()) : A::mk(col[r]);
  }
  auto load_v = [&](int k) {
    const int kc = j0 + k, blo = (kc - j0) >> 5;
    const Z* v = V + (long long)kc * p.ldv;
#pragma unroll
    for (int q = 0; q < BQR_QW; ++q) {
      const int blk = w + NWc * q;
      if (blk < blo || blk >= nblk) continue;
      const int r = j0 + lane + 32 * blk;
      vn[q] = (r < kc || r >= N) ? A::zero() : (r == kc ? A::one() : v[r]);
    }
  };
  load_v(p.conj_tau ? 0 : nb - 1);
  int par = 0;  // parity of the reduction buffer: flips once per barrier
  for (int kk = 0; kk < nb; ++kk) {
    const int k = p.conj_tau ? kk : nb - 1 - kk;
    const int kc = j0 + k, blo = (kc - j0) >> 5;
    Z vr[BQR_QW];
#pragma unroll
    for (int q = 0; q < BQR_QW; ++q) vr[q] = vn[q];
    if (kk + 1 < nb) load_v(p.conj_tau ? kk + 1 : nb - 2 - kk);
    zd t = tau[kc];
    if (t.x == 0.0 && t.y == 0.0) continue;  // uniform over the block
    if (p.conj_tau) t.y = -t.y;
    Z s = A::zero();
#pragma unroll
    for (int q = 0; q < BQR_QW; ++q) {
      const int blk = w + NWc * q;
      if (blk < blo || blk >= nblk) continue;
      s = A::mac(s, A::conj(vr[q]), x[q]);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s = A::add(s, A::shfl_xor(s, o));
    Z tot = s;
    if (NWc > 1) {
      if (lane == 0) red[par][w] = s;
      __syncthreads();
      tot = A::add(A::add(red[par][0], red[par][1]), A::add(red[par][2], red[par][3]));
      par ^= 1;
    }
    const Z f = A::neg(A::mul(A::mk(t), tot));
#pragma unroll
    for (int q = 0; q < BQR_QW; ++q) {
      const int blk = w + NWc * q;
      if (blk < blo || blk >= nblk) continue;
      x[q] = A::mac(x[q], vr[q], f);
    }
  }
  if (fresh)
    for (int r = threadIdx.x; r < j0; r += 32 * NWc) col[r] = zmk(0.0, 0.0);
#pragma unroll
  for (int q = 0; q < BQR_QW; ++q) {
    const int blk = w + NWc * q, r = j0 + lane + 32 * blk;
    if (blk < nblk && r < N) col[r] = A::wide(x[q]);
  }
}

// Four warps per column while the launch's columns leave sub-partitions idle (latency),
// one warp per column once they fill the GPU (fewer reduction instructions per flop).
template <class A>
static inline void bqr_apply(const BQRApply& ap, dim3 grid, cudaStream_t st) {
  const int rows = ap.N - ap.j0;
  const long long cols = (long long)grid.x * grid.y;
  if (cols >= 4 * 152 && rows <= 256) {  // (more rows per lane would spill)
    k_bqr_apply<A, 8, 1><<<grid, 32, 0, st>>>(ap);
  } else {
    if (rows <= 256) k_bqr_apply<A, 2, 4><<<grid, 128, 0, st>>>(ap);
    else if (rows <= 512) k_bqr_apply<A, 4, 4><<<grid, 128, 0, st>>>(ap);
    else k_bqr_apply<A, BQR_LROWS / 4, 4><<<grid, 128, 0, st>>>(ap);
  }
}

// R(i, j) /= D(i) for j >= i (QDRP row normalisation); block x == 0 also forms
// det(Q) = prod det(H_i) (unit-modulus factors) and prod R_ii / D_i, then
// normalises the diagonal (the other blocks touch only the strict upper part).
// grid (ceil(N/8), B), 256 threads; dynamic smem: N doubles.
__global__ void __launch_bounds__(256) k_bqr_finish(zd* A, long long lda, long long sA, int N, const zd* tau,
                                                    long long sT, const double* D, long long sD, QRInfo* info) {
  const int b = blockIdx.y, tid = threadIdx.x, lane = tid & 31;
  zd* M = A + b * sA;
  const double* Db = D + b * sD;
  extern __shared__ double invD[];
  for (int i = tid; i < N; i += 256) invD[i] = bqr_rcp(Db[i]);
  __syncthreads();
  if (blockIdx.x == 0) {
    __shared__ zd pq[256], pr[256];
    zd q = zmk(1.0, 0.0), r = zmk(1.0, 0.0);
    for (int i = tid; i < N; i += 256) {
      const zd z = tau[b * sT + i];
      if (z.x != 0.0 || z.y != 0.0) {
        const double iX = 1.0 / zabs(z);
        const zd h = zsub(zmk(1.0, 0.0), zscale(zscale(z, iX), 2.0 * z.x * iX));
        q = zmul(q, zscale(h, 1.0 / zabs(h)));
      }
      r = zmul(r, zscale(M[i + (long long)i * lda], invD[i]));
    }
    pq[tid] = q; pr[tid] = r;
    __syncthreads();
    for (int s = 128; s > 0; s >>= 1) {
      if (tid < s) { pq[tid] = zmul(pq[tid], pq[tid + s]); pr[tid] = zmul(pr[tid], pr[tid + s]); }
      __syncthreads();
    }
    if (tid == 0) { info[b].detQ = pq[0]; info[b].prodR = pr[0]; }
    for (int i = tid; i < N; i += 256) M[i + (long long)i * lda] = zscale(M[i + (long long)i * lda], invD[i]);
  }
  const int c = blockIdx.x * 8 + (tid >> 5);
  if (c >= N) return;
  zd* col = M + (long long)c * lda;
  for (int r = lane; r < c; r += 32) col[r] = zscale(col[r], invD[r]);
}

// ---------------------------------------------------------------------------------------
// Exact ZGEQP3 (ZLAQP2: dynamic column pivoting with norm downdates,
// Prog/QDRP_decompose_mod.F90:60-101) on one thread-block cluster per matrix.
// Rows are dealt cyclically to the CL CTAs (row i -> CTA i % CL, local row i / CL)
// and kept in shared memory.  Per step j one distributed-shared-memory exchange
// carries, for every column c >= j, the CTA's partial sum_{i>j} conj(a_ij) a_ic
// (c == j: sum |a_ij|^2) and the pivot row; every CTA then holds the same totals,
// applies the reflector to its rows, and downdates its own copy of the column
// norms (identical in all CTAs: same inputs, same summation order), so the pivot
// search needs no exchange.  A column whose downdate loses accuracy (ZLAQP2's
// tol3z test) gets its norm recomputed through one more exchange.  Norms are kept
// squared (the pivot order is the same, the downdate becomes a subtraction).
// Outputs as k_qrp before normalisation: R above, reflectors below, tau, jpvt,
// D = |R_jj|, info.psign; k_bqr_finish then normalises and forms the products.
// GROWS = true keeps each CTA's rows in a global workspace (Arows, one nrl x N block per
// CTA, L2-resident) instead of shared memory, for matrices whose rows do not fit a
// cluster's shared memory (CGR2_2's 2N system at N_dim = 288: 36 rows x 576 columns per
// CTA); the exchange arrays stay in shared memory, and the arithmetic and its order are
// the same as with the rows in shared memory.
struct QRRowsParams {
  const zd* Ain;             // input (may equal A)
  zd* A; long long lda, sA;  // output: R above the diagonal, reflectors below (FP64)
  void* Araw;                // optional: the same in the kernel's arithmetic (for k_bqr_apply)
  int N;
  const double* colscale; long long sCS;
  zd* tau; long long sT;
  int* jpvt; long long sP;
  double* D; long long sD;
  QRInfo* info;
  void* Arows;               // GROWS: workspace of B x CL x nrl x N values of the kernel's arithmetic
  int two_pass;              // 1: every step applies its reflector and forms the next sums in separate passes
};

static inline size_t qrr_smem_bytes(int N, int CL, bool grows = false) {
  const size_t nrl = (size_t)((N + CL - 1) / CL);
  const size_t npad = (size_t)((N + 1) & ~1);  // keeps the 16-byte arrays after it aligned
  return (grows ? 0 : nrl * N * 16) + 6ull * N * 16 + 2ull * N * 8 + npad * 8 + (size_t)N * sizeof(int) + nrl * 16 +
         64;
}
// Elements of the GROWS workspace per matrix.
static inline size_t qrr_rows_elems(int N, int CL) { return (size_t)CL * ((N + CL - 1) / CL) * N; }

template <class Z>
ALF_DEV Z dsm_ld16(uint32_t addr) {  // 16-byte value from a peer CTA's shared memory
  const double v[2] = {dsmem_ld_f64(addr), dsmem_ld_f64(addr + 8)};
  Z z;
  memcpy(&z, v, 16);
  return z;
}

// Lanes ci, ci + cpw, ci + 2 cpw, ... (cpw = 32 >> lk): the 1 << lk threads that share one
// column in the K-threads-per-column mappings of k_qrp_rows.
ALF_DEV unsigned qrr_gmask(int lk, int ci) {
  const int cpw = 32 >> lk;
  unsigned m = 0;
  for (int t = 0; t < (1 << lk); ++t) m |= 1u << (t * cpw);
  return m << ci;
}

template <class Z>
ALF_DEV Z qrr_shfl_xor(Z v, int o, unsigned m) {  // 16-byte value, xor shuffle among the lanes of m
  static_assert(sizeof(Z) == 16, "16-byte values");
  unsigned w[4];
  memcpy(w, &v, 16);
#pragma unroll
  for (int i = 0; i < 4; ++i) w[i] = __shfl_xor_sync(m, w[i], o);
  memcpy(&v, w, 16);
  return v;
}

// Sum over the peers q = s, s + K, ... < CL (K = 1 << lk) of the 16-byte values at `a` in
// their shared memory, four loads in flight.
template <class A>
ALF_DEV typename A::Z qrr_peer_sum(const typename A::Z* a, int s, int lk, int CL) {
  typedef typename A::Z Z;
  Z a0 = A::zero(), a1 = a0, a2 = a0, a3 = a0;
  const int K = 1 << lk, nq = (CL - s + K - 1) >> lk;
  int u = 0;
  for (; u + 3 < nq; u += 4) {
    const Z v0 = dsm_ld16<Z>(dsmem_addr(a, s + (u << lk)));
    const Z v1 = dsm_ld16<Z>(dsmem_addr(a, s + ((u + 1) << lk)));
    const Z v2 = dsm_ld16<Z>(dsmem_addr(a, s + ((u + 2) << lk)));
    const Z v3 = dsm_ld16<Z>(dsmem_addr(a, s + ((u + 3) << lk)));
    a0 = A::add(a0, v0); a1 = A::add(a1, v1);
    a2 = A::add(a2, v2); a3 = A::add(a3, v3);
  }
  for (; u < nq; ++u) a0 = A::add(a0, dsm_ld16<Z>(dsmem_addr(a, s + (u << lk))));
  return A::add(A::add(a0, a1), A::add(a2, a3));
}

template <class A>
ALF_DEV void qrr_argmax(typename A::R& v, int& i) {  // warp argmax, first index on ties
  for (int o = 16; o > 0; o >>= 1) {
    const typename A::R ov = A::rshfl_xor(v, o);
    const int oi = __shfl_xor_sync(0xffffffffu, i, o);
    if (A::gt(ov, v) || (!A::gt(v, ov) && oi < i)) { v = ov; i = oi; }
  }
}

// Arithmetic A: ArD (FP64) or ArF (double-float).  A squared norm of -1 marks a column
// whose norm is recomputed in the extra exchange of the step.
// Column scales: FP64 multiplies A(:,c) by colscale_c on load, like QDRP's caller.
// Double-float has FP32's exponent range, and the UDV scales reach far beyond it, so
// ArF factors the unscaled columns instead: with the same pivots QR(U D) = Q (R_U D)
// (a Householder reflector does not change when its column is scaled), so only the
// pivot keys ||U_c|| d_c (FP64), D and the R output carry the scales.
template <class A, bool GROWS = false>
__global__ void __launch_bounds__(256) k_qrp_rows(QRRowsParams p) {
  typedef typename A::Z Z;
  typedef typename A::R R;
  const unsigned rank = cluster_ctarank(), CL = cluster_nctarank();
  const int b = blockIdx.y, N = p.N, tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int nrl = (N + (int)CL - 1) / (int)CL;
  const int nmine = (N - (int)rank + (int)CL - 1) / (int)CL;  // rows rank, rank+CL, ...
  extern __shared__ __align__(16) unsigned char qrr_raw[];
  // [nrl][N] row-major: Ar[il*N + c] = A(rank + il*CL, c), in shared memory or the workspace
  Z* Ar = GROWS ? reinterpret_cast<Z*>(p.Arows) + ((size_t)b * CL + rank) * (size_t)nrl * N
                : reinterpret_cast<Z*>(qrr_raw);
  Z* xs = GROWS ? reinterpret_cast<Z*>(qrr_raw) : Ar + (size_t)nrl * N;  // [2][N] partial sums (read remotely)
  Z* xr = xs + 2 * N;                     // [2][N] pivot row (owner)
  Z* tot = xr + 2 * N;                    // [N]
  Z* prow = tot + N;                      // [N]
  R* vn1 = reinterpret_cast<R*>(prow + N);
  R* vn2 = vn1 + N;
  double* cs = reinterpret_cast<double*>(vn2 + N);  // [N] column scales (ArF), padded to even length
  Z* vsh = reinterpret_cast<Z*>(cs + ((N + 1) & ~1));  // [nrl], 16-byte aligned
  int* jp = reinterpret_cast<int*>(vsh + nrl);
  constexpr bool sep = A::kDoubleFloat;
  const bool scaled = p.colscale != nullptr;
  __shared__ R s_bv[8];
  __shared__ double s_bvd[8];
  __shared__ int s_bi[8], s_pv, s_cnt;
  __shared__ Z s_zb, s_zt, s_zs;
  __shared__ bool s_triv;
  const R tol3z = A::mkr(1.0536712127723509e-08);  // sqrt(dlamch('Epsilon'))
  const R mone = A::mkr(-1.0);
  zd* Aout = p.A + b * p.sA;
  const long long lda = p.lda;

  for (long long e = tid; e < (long long)nmine * N; e += 256) {
    const int il = (int)(e / N), c = (int)(e % N);
    zd v = p.Ain[b * p.sA + (rank + (long long)il * CL) + c * lda];
    if (scaled && !sep) v = zscale(v, p.colscale[b * p.sCS + c]);
    Ar[(size_t)il * N + c] = A::mk(v);
  }
  for (int c = tid; c < N; c += 256) cs[c] = (scaled && sep) ? fabs(p.colscale[b * p.sCS + c]) : 1.0;
  __syncthreads();
  // initial column norms: exchange 0
  for (int c = tid; c < N; c += 256) {
    R s0 = A::rzero(), s1 = A::rzero();
    int il = 0;
    for (; il + 1 < nmine; il += 2) {
      s0 = A::radd(s0, A::abs2(Ar[(size_t)il * N + c]));
      s1 = A::radd(s1, A::abs2(Ar[(size_t)(il + 1) * N + c]));
    }
    if (il < nmine) s0 = A::radd(s0, A::abs2(Ar[(size_t)il * N + c]));
    xs[c] = A::mkz(A::radd(s0, s1), A::rzero());
    jp[c] = c + 1;
  }
  cluster_sync();
  for (int c = tid; c < N; c += 256) {
    Z s[4] = {A::zero(), A::zero(), A::zero(), A::zero()};
#pragma unroll
    for (int q = 0; q < 16; ++q)
      if (q < (int)CL) s[q & 3] = A::add(s[q & 3], dsm_ld16<Z>(dsmem_addr(&xs[c], q)));
    const R nrm2 = A::re(A::add(A::add(s[0], s[1]), A::add(s[2], s[3])));
    vn1[c] = nrm2; vn2[c] = nrm2;
  }
  int par = 1;
  __syncthreads();

  // Pivot search over the norms vn1[j0..N): the first maximum (times the column scales, ArF).
  auto find_pivot = [&](int j0) -> int {
      if (sep && scaled) {
        double bv = -1.0;
        int bi = N;
        for (int c = j0 + tid; c < N; c += 256) {
          const double v = sqrt(A::rwide(vn1[c])) * cs[c];
          if (v > bv) { bv = v; bi = c; }
        }
        qrr_argmax<ArD>(bv, bi);
        if (lane == 0) { s_bvd[warp] = bv; s_bi[warp] = bi; }
        __syncthreads();
        if (tid == 0) {
          double v = s_bvd[0];
          int i = s_bi[0];
          for (int w = 1; w < 8; ++w)
            if (s_bvd[w] > v || (s_bvd[w] == v && s_bi[w] < i)) { v = s_bvd[w]; i = s_bi[w]; }
          s_pv = (i >= j0 && i < N) ? i : j0;  // NaN norms: keep the column in place
        }
      } else if (!sep) {
        // FP64 norms are >= 0: they order like their IEEE bit patterns, compared on the integer
        // pipes (NaN maps below every norm, so it is never chosen)
        long long bv = -1;
        int bi = N;
        for (int c = j0 + tid; c < N; c += 256) {
          long long v = __double_as_longlong(A::rwide(vn1[c]));
          if ((v & 0x7fffffffffffffffll) > 0x7ff0000000000000ll) v = -1;  // NaN
          if (v == (long long)0x8000000000000000ull) v = 0;                  // -0 ranks as +0
          if (v > bv) { bv = v; bi = c; }
        }
        for (int o = 16; o > 0; o >>= 1) {
          const long long ov = __shfl_xor_sync(0xffffffffu, bv, o);
          const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
          if (ov > bv || (ov == bv && oi < bi)) { bv = ov; bi = oi; }
        }
        if (lane == 0) { s_bi[warp] = bi; s_bvd[warp] = __longlong_as_double(bv); }
        __syncthreads();
        if (tid == 0) {
          long long v = __double_as_longlong(s_bvd[0]);
          int i = s_bi[0];
          for (int w = 1; w < 8; ++w) {
            const long long u = __double_as_longlong(s_bvd[w]);
            if (u > v || (u == v && s_bi[w] < i)) { v = u; i = s_bi[w]; }
          }
          s_pv = (i >= j0 && i < N) ? i : j0;
        }
      } else {
        R bv = mone;
        int bi = N;
        for (int c = j0 + tid; c < N; c += 256) {
          const R v = vn1[c];
          if (A::gt(v, bv)) { bv = v; bi = c; }
        }
        qrr_argmax<A>(bv, bi);
        if (lane == 0) { s_bv[warp] = bv; s_bi[warp] = bi; }
        __syncthreads();
        if (tid == 0) {
          R v = s_bv[0];
          int i = s_bi[0];
          for (int w = 1; w < 8; ++w)
            if (A::gt(s_bv[w], v) || (!A::gt(v, s_bv[w]) && s_bi[w] < i)) { v = s_bv[w]; i = s_bi[w]; }
          s_pv = (i >= j0 && i < N) ? i : j0;  // NaN norms: keep the column in place
        }
      }
      __syncthreads();
      return s_pv;
  };
  // Exchange columns a and pv of the own rows, the permutation, norms, scales and (with_f) the
  // per-column update factors held in tot.
  auto swap_cols = [&](int a, int pv, bool with_f) {
    if (pv == a) return;
    for (int il = tid; il < nmine; il += 256) {
      const Z t = Ar[(size_t)il * N + pv];
      Ar[(size_t)il * N + pv] = Ar[(size_t)il * N + a];
      Ar[(size_t)il * N + a] = t;
    }
    if (tid == 0) {
      const int tj = jp[pv]; jp[pv] = jp[a]; jp[a] = tj;
      vn1[pv] = vn1[a]; vn2[pv] = vn2[a];
      const double ts = cs[pv]; cs[pv] = cs[a]; cs[a] = ts;
      if (with_f) { const Z tf = tot[pv]; tot[pv] = tot[a]; tot[a] = tf; }
    }
    __syncthreads();
  };
  // K = 1 << lk threads per column when few columns remain (rows interleaved, xor-shuffle sums), so
  // the FP64 work spreads over all four sub-partitions.
  auto kmap = [&](int j0, int il0j) {
    int lk = 0;
    while (lk < 4 && ((N - j0) << (lk + 1)) <= 256 && (1 << lk) < nmine - il0j) ++lk;
    return lk;
  };
  // first own row > j0
  auto first_row = [&](int j0) { return (j0 >= (int)rank) ? (j0 - (int)rank) / (int)CL + 1 : 0; };

  // Step j needs the pivot of column j in place and the partial sums of its columns published.
  // Step j normally ends with one pass over its rows that applies its reflector to the trailing
  // columns and, in the same pass, forms step j + 1's partial sums with the updated values
  // (step j + 1's pivot is chosen first: its norms need only the updated pivot row).  A step
  // whose norm downdates need a recomputation applies its reflector alone and the next step
  // starts from its own pivot search.
  bool pre = false;
  for (int j = 0; j < N; ++j) {
    const unsigned owner = (unsigned)(j % (int)CL);
    const int ilj = j / (int)CL;
    const int il0 = first_row(j);
    const int ncol = N - j;
    if (!pre) {
      swap_cols(j, find_pivot(j), false);
      // partials over own rows i > j; the owner of row j publishes it
      Z* xsp = xs + par * N;
      Z* xrp = xr + par * N;
      const int lk = kmap(j, il0);
      const int K = 1 << lk, cpw = 32 >> lk, s = lane / cpw, ci = lane % cpw;
      const unsigned gm = qrr_gmask(lk, ci);
      for (int c = j + warp * cpw + ci; c < N; c += 8 * cpw) {
        Z s0 = A::zero(), s1 = s0;
        int il = il0 + s;
        for (; il + K < nmine; il += 2 * K) {
          s0 = A::mac(s0, A::conj(Ar[(size_t)il * N + j]), Ar[(size_t)il * N + c]);
          s1 = A::mac(s1, A::conj(Ar[(size_t)(il + K) * N + j]), Ar[(size_t)(il + K) * N + c]);
        }
        if (il < nmine) s0 = A::mac(s0, A::conj(Ar[(size_t)il * N + j]), Ar[(size_t)il * N + c]);
        Z acc = A::add(s0, s1);
        for (int o = cpw; o < 32; o <<= 1) acc = A::add(acc, qrr_shfl_xor(acc, o, gm));
        if (s == 0) {
          xsp[c] = acc;
          if (rank == owner) xrp[c] = Ar[(size_t)ilj * N + c];
        }
      }
    }
    pre = false;
    Z* xsp = xs + par * N;
    Z* xrp = xr + par * N;
    cluster_sync();
    {
      int l4 = 0;
      while (l4 < 4 && (ncol << (l4 + 1)) <= 256) ++l4;
      const int cpw = 32 >> l4, s = lane / cpw, ci = lane % cpw;
      const unsigned gm = qrr_gmask(l4, ci);
      for (int c = j + warp * cpw + ci; c < N; c += 8 * cpw) {
        Z acc = qrr_peer_sum<A>(&xsp[c], s, l4, (int)CL);
        for (int o = cpw; o < 32; o <<= 1) acc = A::add(acc, qrr_shfl_xor(acc, o, gm));
        if (s == 0) {
          tot[c] = acc;
          prow[c] = dsm_ld16<Z>(dsmem_addr(&xrp[c], owner));
        }
      }
    }
    par ^= 1;
    __syncthreads();
    // ZLARFG on (alpha, x), x = A(j+1:N, j), and v = scal x over own rows, by warp 0 only
    // (each FP64 instruction occupies its sub-partition ~76 cycles; redundant copies in
    // every warp would multiply that)
    if (warp == 0) {
      const Z alpha = prow[j];
      const R xn2 = A::re(tot[j]);
      const bool triv = A::rzero_p(xn2) && A::rzero_p(A::im(alpha));
      R be = A::re(alpha);
      Z tt = A::zero(), sc = A::zero();
      if (!triv) {
        be = A::rneg(A::rcopysign(A::rsqrt_(A::radd(A::abs2(alpha), xn2)), A::re(alpha)));
        const R ib = A::rrcp(be);
        tt = A::mkz(A::mulr(A::rsub(be, A::re(alpha)), ib), A::rneg(A::mulr(A::im(alpha), ib)));
        sc = A::rcp(A::mkz(A::rsub(A::re(alpha), be), A::im(alpha)));
      }
      for (int il = il0 + lane; il < nmine; il += 32) vsh[il] = A::mul(sc, Ar[(size_t)il * N + j]);
      if (lane == 0) { s_zb = A::mkz(be, A::rzero()); s_zt = tt; s_zs = sc; s_triv = triv; }
    }
    __syncthreads();
    const Z alpha = prow[j];
    const bool trivial = s_triv;
    const R beta = A::re(s_zb);
    const Z t = s_zt, scal = s_zs;
    // Per column c > j (scalars only): the update factor f = conj(tau) (a_jc + conj(scal) x_c)
    // (kept in tot[c]), the updated pivot-row entry (written by its owner), and ZGEQP3's norm
    // downdate.  The norms are kept squared, so the downdate vn1 *= sqrt(max(0, 1 - (|a|/vn1)^2))
    // and the recompute test (vn1/vn2)^2 max(0, 1 - (|a|/vn1)^2) <= tol3z need no division or
    // square root.  Then the reflector into column j.
    int need = 0;
    for (int c = j + 1 + tid; c < N; c += 256) {
      Z anew = prow[c], f = A::zero();
      if (!trivial) {
        f = A::mul(A::conj(t), A::mac(prow[c], A::conj(scal), tot[c]));
        anew = A::sub(anew, f);
        if (rank == owner) Ar[(size_t)ilj * N + c] = anew;
      }
      tot[c] = f;
      const R v1 = vn1[c];
      if (!A::rzero_p(v1)) {
        const R rest = A::rmax0(A::rsub(v1, A::abs2(anew)));
        if (!A::gt(rest, A::mulr(tol3z, vn2[c]))) {
          if (j < N - 1) { need = 1; vn1[c] = mone; }  // recomputed below
          else { vn1[c] = A::rzero(); vn2[c] = A::rzero(); }
        } else {
          vn1[c] = rest;
        }
      }
    }
    if (!trivial) {
      for (int il = il0 + tid; il < nmine; il += 256) Ar[(size_t)il * N + j] = vsh[il];
      if (rank == owner && tid == 0) Ar[(size_t)ilj * N + j] = A::mkz(beta, A::rzero());
    }
    if (rank == owner && tid == 0) {
      p.tau[b * p.sT + j] = A::wide(t);
      p.D[b * p.sD + j] = (trivial ? sqrt(A::rwide(A::abs2(alpha))) : fabs(A::rwide(beta))) * cs[j];
    }
    const bool recompute = __syncthreads_or(need);
    if (recompute || j + 1 >= N || p.two_pass) {
      // H^H on the columns c > j alone: a_c -= v f_c over own rows > j
      if (!trivial) {
        const int lk = kmap(j, il0);
        const int K = 1 << lk, cpw = 32 >> lk, s = lane / cpw, ci = lane % cpw;
        for (int c = j + 1 + warp * cpw + ci; c < N; c += 8 * cpw) {
          const Z nf = A::neg(tot[c]);
          for (int il = il0 + s; il < nmine; il += K)
            Ar[(size_t)il * N + c] = A::mac(Ar[(size_t)il * N + c], vsh[il], nf);
        }
      }
      __syncthreads();
      if (recompute) {
        // exact norms of the flagged columns over rows > j (post-update)
        Z* xq = xs + par * N;
        for (int c = j + 1 + tid; c < N; c += 256) {
          R s0 = A::rzero();
          if (A::rneg_p(vn1[c]))
            for (int il = il0; il < nmine; ++il) s0 = A::radd(s0, A::abs2(Ar[(size_t)il * N + c]));
          xq[c] = A::mkz(s0, A::rzero());
        }
        cluster_sync();
        for (int c = j + 1 + tid; c < N; c += 256) {
          if (!A::rneg_p(vn1[c])) continue;
          Z sq[4] = {A::zero(), A::zero(), A::zero(), A::zero()};
#pragma unroll
          for (int q = 0; q < 16; ++q)
            if (q < (int)CL) sq[q & 3] = A::add(sq[q & 3], dsm_ld16<Z>(dsmem_addr(&xq[c], q)));
          const R nrm2 = A::re(A::add(A::add(sq[0], sq[1]), A::add(sq[2], sq[3])));
          vn1[c] = nrm2; vn2[c] = nrm2;
        }
        par ^= 1;
        __syncthreads();
      }
      continue;
    }
    // step j + 1's pivot (the norms are final), then one pass: the update of step j and the
    // partial sums of step j + 1 over the updated values
    const int j1 = j + 1;
    swap_cols(j1, find_pivot(j1), true);
    const unsigned owner1 = (unsigned)(j1 % (int)CL);
    const int ilj1 = j1 / (int)CL;
    const int il01 = first_row(j1);
    if (!trivial) {  // step j + 1's pivot column first: every other column's sums read it
      const Z nf = A::neg(tot[j1]);
      for (int il = il0 + tid; il < nmine; il += 256)
        Ar[(size_t)il * N + j1] = A::mac(Ar[(size_t)il * N + j1], vsh[il], nf);
    }
    __syncthreads();
    {
      Z* xsp1 = xs + par * N;
      Z* xrp1 = xr + par * N;
      const int lk = kmap(j1, il01);
      const int K = 1 << lk, cpw = 32 >> lk, s = lane / cpw, ci = lane % cpw;
      const unsigned gm = qrr_gmask(lk, ci);
      for (int c = j1 + warp * cpw + ci; c < N; c += 8 * cpw) {
        const bool upd = !trivial && c > j1;
        const Z nf = A::neg(tot[c]);
        Z s0 = A::zero(), s1 = s0;
        int il = il0 + s;
        for (; il + K < nmine; il += 2 * K) {
          Z v0 = Ar[(size_t)il * N + c], v1 = Ar[(size_t)(il + K) * N + c];
          if (upd) {
            v0 = A::mac(v0, vsh[il], nf);
            v1 = A::mac(v1, vsh[il + K], nf);
            Ar[(size_t)il * N + c] = v0;
            Ar[(size_t)(il + K) * N + c] = v1;
          }
          if (il >= il01) s0 = A::mac(s0, A::conj(Ar[(size_t)il * N + j1]), v0);
          s1 = A::mac(s1, A::conj(Ar[(size_t)(il + K) * N + j1]), v1);  // il + K > il0 >= il01 - 1
        }
        if (il < nmine) {
          Z v0 = Ar[(size_t)il * N + c];
          if (upd) {
            v0 = A::mac(v0, vsh[il], nf);
            Ar[(size_t)il * N + c] = v0;
          }
          if (il >= il01) s0 = A::mac(s0, A::conj(Ar[(size_t)il * N + j1]), v0);
        }
        Z acc = A::add(s0, s1);
        for (int o = cpw; o < 32; o <<= 1) acc = A::add(acc, qrr_shfl_xor(acc, o, gm));
        __syncwarp(gm);  // the group's updates of row j + 1 are visible to its publishing lane
        if (s == 0) {
          xsp1[c] = acc;
          if (rank == owner1) xrp1[c] = Ar[(size_t)ilj1 * N + c];
        }
      }
    }
    pre = true;
  }
  Z* raw = p.Araw ? reinterpret_cast<Z*>(p.Araw) + b * p.sA : nullptr;
  for (long long e = tid; e < (long long)nmine * N; e += 256) {
    const int il = (int)(e / N), c = (int)(e % N);
    const long long g = (rank + (long long)il * CL) + c * lda;
    const Z v = Ar[(size_t)il * N + c];
    const long long i = rank + (long long)il * CL;
    Aout[g] = (i <= c) ? zscale(A::wide(v), cs[c]) : A::wide(v);  // R part carries the scales
    if (raw) raw[g] = v;
  }
  if (rank == 0) {
    if (tid == 0) s_cnt = 0;
    __syncthreads();
    int cnt = 0;
    for (int c = tid; c < N; c += 256) {
      const int sc = jp[c];
      for (int i = 0; i < c; ++i) cnt += jp[i] > sc;
      p.jpvt[b * p.sP + c] = sc;
    }
    atomicAdd(&s_cnt, cnt & 1);
    __syncthreads();
    if (tid == 0) p.info[b].psign = (s_cnt & 1) ? -1 : 1;
  }
  cluster_sync();  // no CTA leaves while its shared memory may still be read
}


// ---------------------------------------------------------------------------------------
// Explicit Q in compact-WY form (the mixed form's ZUNGQR on the tensor-core GEMM).  Panel
// of w <= 32 reflectors starting at column j0: H_j0 ... H_{j0+w-1} = I - V T V^H
// (ZLARFT forward / columnwise), Q[:, j0:] <- Q[:, j0:] - (V T) (V^H Q[:, j0:]).
// ---------------------------------------------------------------------------------------

// Q = I for every matrix.  grid (ceil(NN/256), B)
__global__ void k_bqr_eye(zd* Q, int N, long long sQ) {
  const long long NN = (long long)N * N, e = blockIdx.x * 256ll + threadIdx.x;
  if (e >= NN) return;
  Q[blockIdx.y * sQ + e] = zmk((e % N) == (e / N) ? 1.0 : 0.0, 0.0);
}

// T (w x w, upper triangular, ld 32) of one panel from its Gram matrix Gm = V^H V (ld 32) and
// tau: T(i,i) = tau_i; T(0:i, i) = T(0:i, 0:i) (-tau_i Gm(0:i, i)).  One CTA of 256 threads
// per matrix, T in shared memory: warps 1..7 split the triangular mat-vec of each step by
// columns, warp 0 forms z and sums the partials (an FP64 instruction occupies a warp ~64
// cycles, so the serial chain is kept short).
__global__ void __launch_bounds__(256) k_bqr_larft(const zd* Gm, const zd* tau, long long sT, int j0, int w, zd* T) {
  __shared__ zd ts[32][33];  // ts[l][i] = T(l, i)
  __shared__ zd zs[32];
  __shared__ zd part[8][32];
  const int b = blockIdx.x, tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const zd* g = Gm + (long long)b * 32 * 32;
  const zd* tb = tau + b * sT + j0;
  for (int e = tid; e < 32 * 32; e += 256) ts[e % 32][e / 32] = zmk(0.0, 0.0);
  __syncthreads();
  for (int i = 0; i < w; ++i) {
    const zd ti = tb[i];
    if (warp == 0 && lane < i) zs[lane] = zneg(zmul(ti, g[lane + i * 32]));
    __syncthreads();
    if (warp > 0) {
      zd acc = zmk(0.0, 0.0);
      for (int l2 = warp - 1; l2 < i; l2 += 7)
        if (lane <= l2) acc = zfma(ts[lane][l2], zs[l2], acc);
      part[warp][lane] = acc;
    }
    __syncthreads();
    if (warp == 0) {
      zd s = zmk(0.0, 0.0);
#pragma unroll
      for (int q = 1; q < 8; ++q) s = zadd(s, part[q][lane]);
      ts[lane][i] = lane < i ? s : (lane == i ? ti : zmk(0.0, 0.0));
    }
    __syncthreads();
  }
  for (int e = tid; e < 32 * 32; e += 256) T[(long long)b * 1024 + e] = ts[e % 32][e / 32];
}

// X = V T or V T^H (N x w, stored column-major with ld N in the flush layout [matrix][N][32]),
// V the unit lower trapezoid of the panel (column i: 1 at row j0 + i, F(r, j0 + i) below).
// grid (ceil(N / 8), B), block (32, 8): lane = column i, ty = row.
__global__ void k_bqr_vt(const zd* F, long long ldf, long long sF, const zd* T, int N, int j0, int w, zd* X,
                         long long sX, int adj) {
  __shared__ zd ts[32][33];
  const int b = blockIdx.y, i = threadIdx.x, ty = threadIdx.y;
  for (int e = ty * 32 + i; e < 32 * 32; e += 256) ts[e % 32][e / 32] = T[(long long)b * 1024 + e];
  __syncthreads();
  const int r = blockIdx.x * 8 + ty;
  if (r >= N || i >= w) return;
  const zd* f = F + b * sF;
  zd acc = zmk(0.0, 0.0);
  // adj = 0: X = V T (T upper: l <= i); adj = 1: X = V T^H (T^H lower: l >= i, conj(T(i, l)))
  const int l0 = adj ? i : 0, l1 = adj ? w - 1 : i;
  for (int l = l0; l <= l1; ++l) {
    const int c = j0 + l;
    if (r < c) continue;
    const zd v = (r == c) ? zmk(1.0, 0.0) : f[r + c * ldf];
    acc = zfma(v, adj ? zconj(ts[i][l]) : ts[l][i], acc);
  }
  X[b * sX + r + (long long)i * N] = acc;
}
