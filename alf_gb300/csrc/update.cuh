// Sequential single-vertex Metropolis updates with a delayed (submatrix) update.
//
// Reference: Upgrade2 (Prog/upgrade_mod.F90:105-302) called from WRAPGRUP /
// WRAPGRDO (Prog/Wrapgr_mod.F90:115-147, 198-236), for diagonal single-site
// vertices (Op%N = 1): the Mz and SU(N) Hubbard operators.
//
// Within one time slice the vertex exponentials are diagonal similarity
// transforms: G_ii is unchanged by them and the Sherman-Morrison update
// G <- G - x_i G(:,i) (e_i - G(i,:)), x_i = Delta_i / (1 + Delta_i (1 - G_ii)),
// has the same form in the frame of the slice-start matrix G0, so the scalings
// are applied once at the end of the slice by the hopping GEMMs.
//
// A block of nq consecutive visits touches only the sites Sblk of its
// vertices.  The kernel keeps Ghat = G(Sblk, Sblk) in shared memory and applies
// every accepted Sherman-Morrison update to Ghat only; each visit's ratio is
// then Upgrade2's Mat(1,1) = 1 + Delta (1 - Ghat_jj) read directly.  The effect
// on the full matrix is the Woodbury form of the same updates,
//   G = G0 - G0(:,S) Delta_S Gamma^-1 (E_S - G0(S,:)),
//   Gamma = 1 + (1 - G0(S,S)) Delta_S   (S = accepted sites, in accept order),
// applied by one rank-m GEMM flush; Gamma^-1 is formed by k_flush_w.
//
// T is the storage type of G (double2: complex128, used by both precision
// forms).  Ratios, phases and the Metropolis test are always FP64.
#pragma once
#include "common.cuh"

#define UPD_KMAX 32
#define UPD_THREADS 128

struct VertexDev {
  // per chain: K = F*M entries, index k = nf*M + n
  const int* site;       // P(1), 0-based
  const zd* g;
  const zd* alpha;
  const double* E;       // E(1)
  const int8_t* type;    // 1 or 2
  const zd* Eexp;        // [k][5] = E_exp(1, s) at s+2
  long long sK;          // per-chain stride in entries (F*M)
};

struct UpdParams {
  int N, F, M, L, NSUN;
  int nt1;        // slice, 1-based
  int dir;        // 0: up pass (n = pos), 1: down pass (n = M-1-pos)
  int q0, nq;     // visit positions q0 .. q0+nq-1 of this slice
  int visit_base; // visit index (within the sweep) of position 0 of this slice
  void* G; long long sG;  // [chain][F][N][N] of T
  VertexDev V;
  int8_t* fields;       // [chain][L][M]
  const double* draws; long long sDraws;  // [chain][6*M*L] or null
  const unsigned long long* rngkey;      // [chain]
  const unsigned long long* rngctr;      // [chain] counter of draw 0 of this sweep
  zd* phase;            // [chain]
  int* m_out;           // [chain]
  int* sites_out;       // [chain][UPD_KMAX]  accepted sites, accept order
  zd* delta_out;        // [chain][2][UPD_KMAX] Delta of accepted sites
  long long* cnt;       // [chain][4] n_prop, n_acc, n_prop_eff, n_acc_eff
  int8_t* rec_acc; zd* rec_ratio; long long sRec;
  FieldTables ft;
};

template <typename T> struct CT;
template <> struct CT<double2> {
  static ALF_DEV double2 mk(zd a) { return a; }
  static ALF_DEV zd wide(double2 a) { return a; }
};
template <typename T> ALF_DEV T tmul(T a, T b) { T r; r.x = a.x * b.x - a.y * b.y; r.y = a.x * b.y + a.y * b.x; return r; }
template <typename T> ALF_DEV T tadd(T a, T b) { T r; r.x = a.x + b.x; r.y = a.y + b.y; return r; }

ALF_DEV int nranf3(double r) {
  // nint(r*3 + 0.5) clamped to [1,3] (random_wrap_mod.F90:159-168); no contraction.
  double y = __dadd_rn(__dmul_rn(r, 3.0), 0.5);
  int v = (int)round(y);
  return v < 1 ? 1 : (v > 3 ? 3 : v);
}

// One CTA per chain.  Dynamic shared memory: Ghat[F][UPD_KMAX][UPD_KMAX+1] of T.
template <typename T>
__global__ void __launch_bounds__(UPD_THREADS) k_update_block(UpdParams p) {
  const int c = blockIdx.x;
  const int N = p.N, F = p.F, M = p.M, nq = p.nq;
  extern __shared__ __align__(16) unsigned char upd_raw[];
  T* Gh = reinterpret_cast<T*>(upd_raw);  // Gh[(f*UPD_KMAX + a)*LD + b] = G(site_a, site_b)
  constexpr int LD = UPD_KMAX + 1;
  __shared__ int sites[UPD_KMAX], vtx[UPD_KMAX], s_new[UPD_KMAX], prop[UPD_KMAX];
  __shared__ zd myexp[2][UPD_KMAX], dlt[2][UPD_KMAX], expal[2][UPD_KMAX];
  __shared__ double gr[UPD_KMAX], u2[UPD_KMAX];
  __shared__ zd xfac[2];
  __shared__ int s_acc, s_m;
  __shared__ zd s_phase;

  const T* G = reinterpret_cast<const T*>(p.G) + (long long)c * p.sG;
  const int* site = p.V.site + (long long)c * p.V.sK;
  const zd* gg = p.V.g + (long long)c * p.V.sK;
  const zd* al = p.V.alpha + (long long)c * p.V.sK;
  const double* EE = p.V.E + (long long)c * p.V.sK;
  const int8_t* ty = p.V.type + (long long)c * p.V.sK;
  int8_t* fl = p.fields + (long long)c * p.L * M + (long long)(p.nt1 - 1) * M;

  // Prologue: every visit of the block is known in advance (each vertex is visited once
  // per block, so its old field is the field at block start); all FP64 transcendental
  // work is done here in parallel, off the sequential chain.
  for (int q = threadIdx.x; q < nq; q += blockDim.x) {
    const int pos = p.q0 + q;
    const int n = p.dir == 0 ? pos : M - 1 - pos;
    vtx[q] = n;
    sites[q] = site[n];
    const int v = p.visit_base + pos;
    double u0, u1, uu2;
    if (p.draws) {
      const double* d = p.draws + (long long)c * p.sDraws + 3ll * v;
      u0 = d[0]; u1 = d[1]; uu2 = d[2];
    } else {
      unsigned long long key = p.rngkey[c], ctr = p.rngctr[c] + 3ull * v;
      u0 = alf_uniform(key, ctr); u1 = alf_uniform(key, ctr + 1); uu2 = alf_uniform(key, ctr + 2);
    }
    const int so = fl[n], tp = ty[n];
    const int sn = (tp == 1) ? -so : (int)p.ft.flip[so + 2][nranf3(u0) - 1];
    s_new[q] = sn;
    prop[q] = 1.5 > u1;  // T0_proposal (Wrapgr_mod.F90:123,133); always true
    u2[q] = uu2;
    gr[q] = p.ft.gama[tp - 1][sn + 2] / p.ft.gama[tp - 1][so + 2];
    const double dphi = p.ft.phi[tp - 1][sn + 2] - p.ft.phi[tp - 1][so + 2];
    for (int f = 0; f < F; ++f) {
      const int k = f * M + n;
      const zd Z1 = zscale(gg[k], dphi);
      const zd me = zexp(zscale(Z1, EE[k]));
      myexp[f][q] = me;
      dlt[f][q] = zsub(me, zmk(1.0, 0.0));
      expal[f][q] = zexp(zmul(Z1, al[k]));
    }
  }
  if (threadIdx.x == 0) { s_m = 0; s_phase = p.phase[c]; }
  __syncthreads();
  for (int e = threadIdx.x; e < F * nq * nq; e += blockDim.x) {
    const int f = e / (nq * nq), r = e % (nq * nq), a = r % nq, b = r / nq;
    Gh[(f * UPD_KMAX + a) * LD + b] = G[(long long)f * N * N + sites[a] + (long long)sites[b] * N];
  }
  __syncthreads();

  long long n_prop = 0, n_acc = 0;
  for (int q = 0; q < nq; ++q) {
    if (threadIdx.x == 0) {
      int acc = 0;
      zd R = zmk(0.0, 0.0);
      if (prop[q]) {
        zd D[2];
        for (int f = 0; f < F; ++f) {
          const zd gjj = CT<T>::wide(Gh[(f * UPD_KMAX + q) * LD + q]);
          D[f] = zsub(myexp[f][q], zmul(dlt[f][q], gjj));  // Mat(1,1) = myexp - Z*G(P,P)
          const zd Rf = zmul(D[f], expal[f][q]);
          R = (f == 0) ? Rf : zmul(R, Rf);
        }
        zd Rp = R;
        for (int e = 1; e < p.NSUN; ++e) Rp = zmul(Rp, R);
        R = zscale(Rp, gr[q]);
        const zd ph = s_phase;
        const double weight = fabs(zmul(ph, R).x / ph.x);
        acc = weight > u2[q];
        if (acc) {
          const double ar = sqrt(zmul(R, zconj(R)).x);
          const zd pr = zmul(ph, R);
          s_phase = zmk(pr.x / ar, pr.y / ar);
          for (int f = 0; f < F; ++f) xfac[f] = zdiv(dlt[f][q], D[f]);  // x = Delta / (1 + Delta (1 - G_jj))
        }
      }
      if (p.rec_acc) {
        const int v = p.visit_base + p.q0 + q;
        p.rec_acc[(long long)c * p.sRec + v] = (int8_t)acc;
        p.rec_ratio[(long long)c * p.sRec + v] = R;
      }
      s_acc = acc;
    }
    __syncthreads();
    n_prop += prop[q];
    if (s_acc) {
      ++n_acc;
      // Ghat(a,b) += x Ghat(a,q) Ghat(q,b) for the positions still to be visited (a, b > q)
      const int rem = nq - q - 1;
      for (int e = threadIdx.x; e < F * rem * rem; e += blockDim.x) {
        const int f = e / (rem * rem), r = e % (rem * rem), a = q + 1 + r % rem, b = q + 1 + r / rem;
        const T x = CT<T>::mk(xfac[f]);
        const T gaq = Gh[(f * UPD_KMAX + a) * LD + q];
        const T gqb = Gh[(f * UPD_KMAX + q) * LD + b];
        Gh[(f * UPD_KMAX + a) * LD + b] = tadd(Gh[(f * UPD_KMAX + a) * LD + b], tmul(x, tmul(gaq, gqb)));
      }
      if (threadIdx.x == 0) {
        const int m = s_m;
        p.sites_out[(long long)c * UPD_KMAX + m] = sites[q];
        for (int f = 0; f < F; ++f) p.delta_out[((long long)c * 2 + f) * UPD_KMAX + m] = dlt[f][q];
        s_m = m + 1;
        fl[vtx[q]] = (int8_t)s_new[q];
      }
      __syncthreads();
    }
  }
  if (threadIdx.x == 0) {
    p.m_out[c] = s_m;
    p.phase[c] = s_phase;
    long long* cn = p.cnt + 4ll * c;
    cn[0] += n_prop; cn[1] += n_acc; cn[2] += nq; cn[3] += n_acc;
  }
}

// W = Delta_S Gamma^-1, Gamma = 1 + (1 - G0(S,S)) Delta_S: Gauss-Jordan elimination with
// partial pivoting on [Gamma^T | I] (so the right half becomes Gamma^-T).  One CTA per
// (chain, flavour); W: [chain][2][KMAX][KMAX] row-major (l, l').
template <typename T>
__global__ void __launch_bounds__(256) k_flush_w(const void* Gv, long long sG, int N, int F, const int* m_in,
                                                 const int* sites, const zd* delta, zd* W) {
  const int b = blockIdx.x, c = b / F, f = b % F;
  const int m = m_in[c];
  if (m == 0) return;
  const T* G = reinterpret_cast<const T*>(Gv) + (long long)c * sG + (long long)f * N * N;
  __shared__ zd A[UPD_KMAX][2 * UPD_KMAX + 1];
  __shared__ int st[UPD_KMAX];
  __shared__ zd dl[UPD_KMAX];
  __shared__ int piv;
  __shared__ zd pinv;
  for (int l = threadIdx.x; l < m; l += blockDim.x) {
    st[l] = sites[(long long)c * UPD_KMAX + l];
    dl[l] = delta[((long long)c * 2 + f) * UPD_KMAX + l];
  }
  __syncthreads();
  // A(r, col) = Gamma(col, r) = delta + (delta - G0(s_col, s_r)) Delta_r
  for (int e = threadIdx.x; e < m * m; e += blockDim.x) {
    const int r = e % m, col = e / m;
    const zd g = CT<T>::wide(G[st[col] + (long long)st[r] * N]);
    zd v = zmul(zsub(zmk(col == r ? 1.0 : 0.0, 0.0), g), dl[r]);
    if (col == r) v = zadd(v, zmk(1.0, 0.0));
    A[r][col] = v;
    A[r][m + col] = zmk(r == col ? 1.0 : 0.0, 0.0);
  }
  __syncthreads();
  for (int k = 0; k < m; ++k) {
    if (threadIdx.x == 0) {
      int pv = k;
      double best = A[k][k].x * A[k][k].x + A[k][k].y * A[k][k].y;
      for (int r = k + 1; r < m; ++r) {
        const double v = A[r][k].x * A[r][k].x + A[r][k].y * A[r][k].y;
        if (v > best) { best = v; pv = r; }
      }
      piv = pv;
      pinv = zinv(A[pv][k]);
    }
    __syncthreads();
    const int pv = piv;
    if (pv != k)
      for (int j = threadIdx.x; j < 2 * m; j += blockDim.x) { zd t = A[k][j]; A[k][j] = A[pv][j]; A[pv][j] = t; }
    __syncthreads();
    const zd inv = pinv;
    for (int j = threadIdx.x; j < 2 * m; j += blockDim.x)
      if (j != k) A[k][j] = zmul(A[k][j], inv);
    __syncthreads();
    for (int e = threadIdx.x; e < m * 2 * m; e += blockDim.x) {
      const int r = e / (2 * m), j = e % (2 * m);
      if (r != k && j != k) A[r][j] = zsub(A[r][j], zmul(A[r][k], A[k][j]));
    }
    __syncthreads();
  }
  // Gamma^-1(l, l') = A(l', m + l);  W(l, l') = Delta_l Gamma^-1(l, l')
  for (int e = threadIdx.x; e < m * m; e += blockDim.x) {
    const int l = e / m, l2 = e % m;
    W[(((long long)c * 2 + f) * UPD_KMAX + l) * UPD_KMAX + l2] = zmul(dl[l], A[l2][m + l]);
  }
}

// Flush operands, spread over the GPU:
//   X(:, l) = G0(:, s_l)                                   (k_flush_x: one thread per (row, l))
//   Y(l, :) = sum_l' W(l,l') (e_{s_l'} - G0(s_l', :))      (k_flush_y: one thread per (l, column))
// X: [chain][2][N][KMAX] col-major (ld N); Y: [chain][2][KMAX][N] col-major (ld KMAX), type T.
template <typename T>
__global__ void k_flush_x(const void* Gv, long long sG, int N, int F, const int* m_in, const int* sites, void* Xv) {
  const int b = blockIdx.y, c = b / F, f = b % F;
  const int m = m_in[c];
  const long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (e >= (long long)N * m) return;
  const int row = e % N, l = e / N;
  const int s = sites[(long long)c * UPD_KMAX + l];
  const T* G = reinterpret_cast<const T*>(Gv);
  T* X = reinterpret_cast<T*>(Xv);
  X[((long long)c * 2 + f) * N * UPD_KMAX + row + (long long)l * N] =
      G[(long long)c * sG + (long long)f * N * N + row + (long long)s * N];
}

// block: 32 x 8 threads = (l, column); grid (ceil(N/8), B)
template <typename T>
__global__ void k_flush_y(const void* Gv, long long sG, int N, int F, const int* m_in, const int* sites, const zd* W,
                          void* Yv) {
  const int b = blockIdx.y, c = b / F, f = b % F;
  const int m = m_in[c];
  if (m == 0) return;
  __shared__ zd Ws[UPD_KMAX][UPD_KMAX + 1];
  __shared__ zd gb[8][UPD_KMAX];
  __shared__ int st[UPD_KMAX];
  const int tx = threadIdx.x, ty = threadIdx.y, tid = ty * 32 + tx;
  for (int l = tid; l < m; l += 256) st[l] = sites[(long long)c * UPD_KMAX + l];
  for (int e = tid; e < m * m; e += 256)
    Ws[e / m][e % m] = W[(((long long)c * 2 + f) * UPD_KMAX + e / m) * UPD_KMAX + e % m];
  __syncthreads();
  const int col = blockIdx.x * 8 + ty;
  const T* Gf = reinterpret_cast<const T*>(Gv) + (long long)c * sG + (long long)f * N * N;
  if (col < N && tx < m) {
    const int s = st[tx];
    const zd gv = CT<T>::wide(Gf[s + (long long)col * N]);
    gb[ty][tx] = zsub(zmk(s == col ? 1.0 : 0.0, 0.0), gv);
  }
  __syncthreads();
  if (col < N && tx < m) {
    zd y = zmk(0.0, 0.0);
    for (int l2 = 0; l2 < m; ++l2) y = zadd(y, zmul(Ws[tx][l2], gb[ty][l2]));
    reinterpret_cast<T*>(Yv)[((long long)c * 2 + f) * N * UPD_KMAX + tx + (long long)col * UPD_KMAX] = CT<T>::mk(y);
  }
}

template <typename T> constexpr size_t upd_smem_bytes() { return 2 * UPD_KMAX * (UPD_KMAX + 1) * sizeof(T); }
