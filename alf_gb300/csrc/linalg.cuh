// Stabilisation kernels: column-pivoted Householder QR (ZGEQP3 / ZLAQP2
// semantics, as called by QDRP_decompose, Prog/QDRP_decompose_mod.F90:60-101),
// explicit Q (ZUNGQR / ZUNG2R), multi-RHS triangular solves (ZTRSM) and small
// helpers.  Each QR / Q-formation runs on one thread-block cluster: columns
// are dealt cyclically to the CTAs, the pivot argmax is reduced through
// distributed shared memory, and barrier.cluster separates the steps.
#pragma once
#include "common.cuh"

#define QR_THREADS 256

struct QRInfo {  // per matrix, written by the QR kernel
  zd detQ;       // prod_i det(H_i) = prod (1 - 2 (tau/|tau|) Re(tau)/|tau|)
  zd prodR;      // prod_i R(i,i) after the QDRP row normalisation
  int psign;     // sign of the column permutation (Pivot_phase, QDRP_decompose_mod.F90:103-126)
  int pad;
};

struct QRParams {
  zd* A; long long lda, sA;  // N x N, in place: R (normalised rows) above, Householder vectors below
  int N;
  zd* tau; long long sT;     // [N]
  int* jpvt; long long sP;   // [N], 1-based like LAPACK
  double* D; long long sD;   // [N] = |R(i,i)|
  double* vn; long long sV;  // [2N] work: vn1, vn2
  const double* colscale; long long sCS;  // optional: A(:,i) *= colscale[i] first (U*D of decompose)
  QRInfo* info;
};

// Squared 2-norm of a complex vector segment, computed by one warp: the plain sum of
// squares (FP64 products only); the scaled form below when that sum over- or underflows.
ALF_DEV double warp_znrm2(const zd* x, int n);
ALF_DEV double warp_znrm2sq(const zd* x, int n) {
  double s = 0.0;
  for (int i = threadIdx.x & 31; i < n; i += 32) s = fma(x[i].x, x[i].x, fma(x[i].y, x[i].y, s));
  s = warp_sum(s);
  if (!(s < 1e300) || (s != 0.0 && s < 1e-290)) {
    const double r = warp_znrm2(x, n);
    s = r * r;
  }
  return s;
}

// Scaled 2-norm of a strided complex vector segment, computed by one warp.
ALF_DEV double warp_znrm2(const zd* x, int n) {
  double mx = 0.0;
  for (int i = threadIdx.x & 31; i < n; i += 32) mx = fmax(mx, fmax(fabs(x[i].x), fabs(x[i].y)));
  mx = warp_max(mx);
  if (mx == 0.0) return 0.0;
  double s = 0.0, inv = 1.0 / mx;
  for (int i = threadIdx.x & 31; i < n; i += 32) {
    double a = x[i].x * inv, b = x[i].y * inv;
    s += a * a + b * b;
  }
  s = warp_sum(s);
  return mx * sqrt(s);
}

__global__ void __launch_bounds__(QR_THREADS) k_qrp(QRParams p) {
  const unsigned rank = cluster_ctarank(), CL = cluster_nctarank();
  const int b = blockIdx.y;
  const int N = p.N;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, NW = QR_THREADS / 32;
  zd* A = p.A + b * p.sA;
  const long long lda = p.lda;
  zd* tau = p.tau + b * p.sT;
  int* jpvt = p.jpvt + b * p.sP;
  double* vn1 = p.vn + b * p.sV;
  double* vn2 = vn1 + N;
  __shared__ double cand_val;
  __shared__ int cand_idx;
  __shared__ double red_v[QR_THREADS / 32];
  __shared__ int red_i[QR_THREADS / 32];
  __shared__ int s_piv;
  extern __shared__ zd vsh[];  // Householder vector of the current step (N entries)
  const double tol3z = 1.0536712127723509e-08;  // sqrt(dlamch('Epsilon'))

  // Prologue: optional column scaling, initial norms, jpvt.
  for (int c = rank + CL * warp; c < N; c += CL * NW) {
    zd* col = A + (long long)c * lda;
    if (p.colscale) {
      double s = p.colscale[b * p.sCS + c];
      for (int r = lane; r < N; r += 32) col[r] = zscale(col[r], s);
      __syncwarp();
    }
    const double nrm2 = warp_znrm2sq(col, N);  // squared norms throughout (same pivot order)
    if (lane == 0) { vn1[c] = nrm2; vn2[c] = nrm2; jpvt[c] = c + 1; }
  }
  cluster_sync();

  for (int j = 0; j < N; ++j) {
    // local argmax of vn1 over owned columns >= j (first index on ties)
    double bv = -1.0;
    int bi = N;
    for (int c = rank + CL * warp; c < N; c += CL * NW) {
      if (c >= j) {
        double v = vn1[c];
        if (v > bv || (v == bv && c < bi)) { bv = v; bi = c; }
      }
    }
    if (lane == 0) { red_v[warp] = bv; red_i[warp] = bi; }
    __syncthreads();
    if (threadIdx.x == 0) {
      double v = -1.0;
      int i = N;
      for (int w = 0; w < NW; ++w)
        if (red_v[w] > v || (red_v[w] == v && red_i[w] < i)) { v = red_v[w]; i = red_i[w]; }
      cand_val = v;
      cand_idx = i;
    }
    cluster_sync();  // B1: candidates published (and previous step's updates visible)
    if (threadIdx.x == 0) {
      double v = -1.0;
      int i = N;
      for (unsigned r = 0; r < CL; ++r) {
        double rv = dsmem_ld_f64(dsmem_addr(&cand_val, r));
        int ri = dsmem_ld_s32(dsmem_addr(&cand_idx, r));
        if (rv > v || (rv == v && ri < i)) { v = rv; i = ri; }
      }
      s_piv = (i >= j && i < N) ? i : j;  // NaN norms: keep the column in place
    }
    __syncthreads();
    const int pv = s_piv;
    const unsigned owner = j % CL;
    if (rank == owner) {
      zd* cj = A + (long long)j * lda;
      if (pv != j) {
        zd* cp = A + (long long)pv * lda;
        for (int r = threadIdx.x; r < N; r += QR_THREADS) { zd t = cp[r]; cp[r] = cj[r]; cj[r] = t; }
        if (threadIdx.x == 0) {
          int t = jpvt[pv]; jpvt[pv] = jpvt[j]; jpvt[j] = t;
          vn1[pv] = vn1[j]; vn2[pv] = vn2[j];
        }
        __syncthreads();
      }
      // ZLARFG on A(j:N, j)
      if (warp == 0) {
        const int nx = N - j - 1;
        const double xn2 = warp_znrm2sq(cj + j + 1, nx);
        zd alpha = cj[j];
        zd t = zmk(0.0, 0.0), scal = zmk(0.0, 0.0);
        double beta = 0.0;
        bool trivial = (xn2 == 0.0 && alpha.y == 0.0);
        if (!trivial) {
          double ar = alpha.x, ai = alpha.y;
          double l3 = sqrt(fma(ar, ar, fma(ai, ai, xn2)));
          if (!(l3 < 1e150)) {  // the scaled form of ZLAPY3 where the squares could overflow
            const double xnorm = sqrt(xn2), w = fmax(fabs(ar), fmax(fabs(ai), xnorm));
            l3 = w * sqrt((ar / w) * (ar / w) + (ai / w) * (ai / w) + (xnorm / w) * (xnorm / w));
          }
          beta = -copysign(l3, ar);
          t = zmk((beta - ar) / beta, -ai / beta);
          scal = zdiv(zmk(1.0, 0.0), zsub(alpha, zmk(beta, 0.0)));
        }
        if (!trivial) {
          for (int r = j + 1 + lane; r < N; r += 32) cj[r] = zmul(scal, cj[r]);
        }
        if (lane == 0) {
          tau[j] = t;
          if (!trivial) cj[j] = zmk(beta, 0.0);
        }
      }
    }
    cluster_sync();  // B2: reflector j visible
    // stage v = (1, A(j+1:N, j)) in shared memory
    {
      const zd* cj = A + (long long)j * lda;
      for (int r = j + threadIdx.x; r < N; r += QR_THREADS) vsh[r] = (r == j) ? zmk(1.0, 0.0) : cj[r];
    }
    __syncthreads();
    const zd ct = zconj(tau[j]);
    for (int c = rank + CL * warp; c < N; c += CL * NW) {
      if (c <= j) continue;
      zd* col = A + (long long)c * lda;
      zd s = zmk(0.0, 0.0);
      if (ct.x != 0.0 || ct.y != 0.0) {
        for (int r = j + lane; r < N; r += 32) s = zfma(zconj(vsh[r]), col[r], s);
        s = warp_zsum(s);
        zd f = zmul(ct, s);
        for (int r = j + lane; r < N; r += 32) col[r] = zsub(col[r], zmul(vsh[r], f));
        __syncwarp();
      }
      // norm downdate (ZLAQP2) on squared norms: vn1^2 (1 - (|a|/vn1)^2) = vn1^2 - |a|^2, and the
      // recompute test (vn1/vn2)^2 max(0, 1 - (|a|/vn1)^2) <= tol3z needs no division
      const double v1 = vn1[c];
      if (v1 != 0.0) {
        const zd a = col[j];
        const double rest = fmax(v1 - fma(a.x, a.x, a.y * a.y), 0.0);
        double nv1 = rest, nv2 = vn2[c];
        if (rest <= tol3z * nv2) {
          if (j < N - 1) { nv1 = warp_znrm2sq(col + j + 1, N - j - 1); nv2 = nv1; }
          else { nv1 = 0.0; nv2 = 0.0; }
        }
        if (lane == 0) { vn1[c] = nv1; vn2[c] = nv2; }
      }
    }
  }
  cluster_sync();
  // D(i) = |R(i,i)|, then normalise rows of R (QDRP_decompose_mod.F90:85-100)
  double* D = p.D + b * p.sD;
  for (int c = rank + CL * warp; c < N; c += CL * NW)
    if (lane == 0) D[c] = zabs(A[c + (long long)c * lda]);
  cluster_sync();
  for (int c = rank + CL * warp; c < N; c += CL * NW) {
    zd* col = A + (long long)c * lda;
    for (int r = lane; r <= c; r += 32) col[r] = zscale(col[r], 1.0 / D[r]);
  }
  cluster_sync();
  if (rank == 0 && threadIdx.x == 0) {
    zd dq = zmk(1.0, 0.0), pr = zmk(1.0, 0.0);
    for (int i = 0; i < N; ++i) {
      pr = zmul(pr, A[i + (long long)i * lda]);
      zd z = tau[i];
      if (z.x != 0.0 || z.y != 0.0) {
        double X = zabs(z);
        zd h = zsub(zmk(1.0, 0.0), zscale(zscale(z, 1.0 / X), 2.0 * z.x / X));
        dq = zmul(dq, zscale(h, 1.0 / zabs(h)));
      }
    }
    // permutation sign by cycle lengths (visited flags reuse the vector buffer)
    int* vis = reinterpret_cast<int*>(vsh);
    for (int i = 0; i < N; ++i) vis[i] = 0;
    int sgn = 1;
    for (int i = 0; i < N; ++i) {
      if (vis[i]) continue;
      int next = i, len = 0;
      while (next >= 0 && next < N && !vis[next]) { vis[next] = 1; len++; next = jpvt[next] - 1; }
      if (len % 2 == 0) sgn = -sgn;
    }
    p.info[b].detQ = dq;
    p.info[b].prodR = pr;
    p.info[b].psign = sgn;
  }
}

// Explicit Q from the Householder vectors in A (ZUNG2R), in place.
struct OrgqrParams {
  zd* A; long long lda, sA;
  const zd* tau; long long sT;
  int N;
};

__global__ void __launch_bounds__(QR_THREADS) k_orgqr(OrgqrParams p) {
  const unsigned rank = cluster_ctarank(), CL = cluster_nctarank();
  const int b = blockIdx.y, N = p.N;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, NW = QR_THREADS / 32;
  zd* A = p.A + b * p.sA;
  const long long lda = p.lda;
  const zd* tau = p.tau + b * p.sT;
  extern __shared__ zd vsh[];
  for (int i = N - 1; i >= 0; --i) {
    const zd* ci = A + (long long)i * lda;
    for (int r = i + threadIdx.x; r < N; r += QR_THREADS) vsh[r] = (r == i) ? zmk(1.0, 0.0) : ci[r];
    cluster_sync();
    const zd ti = tau[i];
    if (rank == (unsigned)(i % CL)) {
      zd* c = A + (long long)i * lda;
      for (int r = threadIdx.x; r < N; r += QR_THREADS) {
        if (r < i) c[r] = zmk(0.0, 0.0);
        else if (r == i) c[r] = zsub(zmk(1.0, 0.0), ti);
        else c[r] = zneg(zmul(ti, vsh[r]));
      }
    }
    if (ti.x != 0.0 || ti.y != 0.0) {
      for (int c = rank + CL * warp; c < N; c += CL * NW) {
        if (c <= i) continue;
        zd* col = A + (long long)c * lda;
        zd s = zmk(0.0, 0.0);
        for (int r = i + lane; r < N; r += 32) s = zfma(zconj(vsh[r]), col[r], s);
        s = warp_zsum(s);
        zd f = zmul(ti, s);
        for (int r = i + lane; r < N; r += 32) col[r] = zsub(col[r], zmul(vsh[r], f));
      }
    }
    __syncthreads();
  }
}

// Multi-RHS triangular solve T x = b, T stored N x N column-major:
// upper (backward substitution) or lower (forward).  RHS vector v has entries
// B[v*vstride + i*estride]; conj_io conjugates on load and store (used for the
// right-sided solves X op(R) = B by working on rows).  One CTA per vector.
struct TrsvParams {
  const zd* T; long long ldt, sT;
  zd* B; long long vstride, estride, sB;
  int N, nvec, lower, conj_io;
  int trans;             // 1: the triangle is conj(T)^T (T(i,j) read as conj(T(j,i)))
  const double* oscale;  // optional: x_i *= oscale[i] after the solve (per batch, stride N)
};

// Dynamic shared memory: 3 N complex values (right-hand side, solution, diagonal
// reciprocals).  Every thread forms x_i itself from the finished right-hand side entry,
// so a row costs one barrier and no serial division.
__global__ void __launch_bounds__(256) k_trsv(TrsvParams p) {
  const int b = blockIdx.y, v = blockIdx.x, N = p.N;
  if (v >= p.nvec) return;
  const zd* T = p.T + b * p.sT;
  zd* x = p.B + b * p.sB + (long long)v * p.vstride;
  extern __shared__ zd xs[];
  zd* xo = xs + N;
  zd* dinv = xo + N;
  auto Tij = [&](int i, int j) -> zd {
    return p.trans ? zconj(T[j + (long long)i * p.ldt]) : T[i + (long long)j * p.ldt];
  };
  for (int i = threadIdx.x; i < N; i += blockDim.x) {
    zd t = x[(long long)i * p.estride];
    xs[i] = p.conj_io ? zconj(t) : t;
    dinv[i] = zinv(Tij(i, i));
  }
  __syncthreads();
  if (!p.lower) {
    for (int i = N - 1; i >= 0; --i) {
      const zd xi = zmul(xs[i], dinv[i]);
      if (threadIdx.x == 0) xo[i] = xi;
      for (int r = threadIdx.x; r < i; r += blockDim.x) xs[r] = zsub(xs[r], zmul(Tij(r, i), xi));
      __syncthreads();
    }
  } else {
    for (int i = 0; i < N; ++i) {
      const zd xi = zmul(xs[i], dinv[i]);
      if (threadIdx.x == 0) xo[i] = xi;
      for (int r = i + 1 + threadIdx.x; r < N; r += blockDim.x) xs[r] = zsub(xs[r], zmul(Tij(r, i), xi));
      __syncthreads();
    }
  }
  for (int i = threadIdx.x; i < N; i += blockDim.x) {
    zd t = xo[i];
    if (p.oscale) t = zscale(t, p.oscale[(long long)b * N + i]);
    x[(long long)i * p.estride] = p.conj_io ? zconj(t) : t;
  }
}

// The same solve for V right-hand sides per CTA (vectors V blockIdx.x .. + V - 1): thread t
// works on vector t % V and rows t / V, t / V + 256 / V, ...; the V threads of a row read the
// same triangle entry (one broadcast load feeds V products) and one barrier per row serves V
// vectors.  Dynamic shared memory: (2 V + 1) N complex values.  Same arithmetic per vector as
// k_trsv.
template <int V>
__global__ void __launch_bounds__(256) k_trsv_v(TrsvParams p) {
  const int b = blockIdx.y, v0 = blockIdx.x * V, N = p.N, tid = threadIdx.x;
  const zd* T = p.T + b * p.sT;
  zd* Bb = p.B + b * p.sB;
  extern __shared__ zd tsm[];
  zd* xs = tsm;            // [V][N]
  zd* xo = xs + V * N;     // [V][N]
  zd* dinv = xo + V * N;   // [N]
  auto Tij = [&](int i, int j) -> zd {
    return p.trans ? zconj(T[j + (long long)i * p.ldt]) : T[i + (long long)j * p.ldt];
  };
  for (int e = tid; e < V * N; e += 256) {
    const int v = e / N, i = e % N;
    zd t = zmk(0.0, 0.0);
    if (v0 + v < p.nvec) {
      t = Bb[(long long)(v0 + v) * p.vstride + (long long)i * p.estride];
      if (p.conj_io) t = zconj(t);
    }
    xs[v * N + i] = t;
  }
  for (int i = tid; i < N; i += 256) dinv[i] = zinv(Tij(i, i));
  __syncthreads();
  const int v = tid % V, r0 = tid / V, rs = 256 / V;
  zd* x = xs + v * N;
  if (!p.lower) {
    for (int i = N - 1; i >= 0; --i) {
      const zd xi = zmul(x[i], dinv[i]);
      if (r0 == 0) xo[v * N + i] = xi;
      for (int r = r0; r < i; r += rs) x[r] = zfms(Tij(r, i), xi, x[r]);
      __syncthreads();
    }
  } else {
    for (int i = 0; i < N; ++i) {
      const zd xi = zmul(x[i], dinv[i]);
      if (r0 == 0) xo[v * N + i] = xi;
      for (int r = i + 1 + r0; r < N; r += rs) x[r] = zfms(Tij(r, i), xi, x[r]);
      __syncthreads();
    }
  }
  for (int e = tid; e < V * N; e += 256) {
    const int vv = e / N, i = e % N;
    if (v0 + vv >= p.nvec) continue;
    zd t = xo[vv * N + i];
    if (p.oscale) t = zscale(t, p.oscale[(long long)b * N + i]);
    Bb[(long long)(v0 + vv) * p.vstride + (long long)i * p.estride] = p.conj_io ? zconj(t) : t;
  }
}
#define TRSV_V 8
static inline size_t trsv_v_smem(int N) { return (size_t)(2 * TRSV_V + 1) * N * 16; }

// out(j, i) = conj(in(i, j)) (or plain transpose), batched, N x N.
__global__ void k_transpose(const zd* in, long long ldi, long long sI, zd* out, long long ldo, long long sO, int N,
                            int conj) {
  __shared__ zd tile[32][33];
  const int b = blockIdx.z;
  const int bx = blockIdx.x * 32, by = blockIdx.y * 32;
  const zd* I = in + b * sI;
  zd* O = out + b * sO;
  for (int k = threadIdx.y; k < 32; k += blockDim.y) {
    int r = bx + threadIdx.x, c = by + k;
    if (r < N && c < N) tile[k][threadIdx.x] = I[r + (long long)c * ldi];
  }
  __syncthreads();
  for (int k = threadIdx.y; k < 32; k += blockDim.y) {
    int r = by + threadIdx.x, c = bx + k;
    if (r < N && c < N) {
      zd v = tile[threadIdx.x][k];
      O[r + (long long)c * ldo] = conj ? zconj(v) : v;
    }
  }
}

// inverse permutation of a 1-based LAPACK pivot vector: inv[jpvt[i]-1] = i
__global__ void k_invperm(const int* jpvt, long long sP, int* inv, long long sI, int N) {
  const int b = blockIdx.y;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += blockDim.x * gridDim.x)
    inv[b * sI + jpvt[b * sP + i] - 1] = i;
}

// 0-based copy of a 1-based pivot vector
__global__ void k_perm0(const int* jpvt, long long sP, int* out, long long sO, int N) {
  const int b = blockIdx.y;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += blockDim.x * gridDim.x)
    out[b * sO + i] = jpvt[b * sP + i] - 1;
}
