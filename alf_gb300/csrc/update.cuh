// Sequential single-vertex Metropolis updates with a delayed (submatrix) update.
//
// Reference: Upgrade2 (Prog/upgrade_mod.F90:105-302) called from WRAPGRUP /
// WRAPGRDO (Prog/Wrapgr_mod.F90:115-147, 198-236), for diagonal single-site
// vertices (Op%N = 1), the Hubbard/Mz and SU(N) Hubbard operators.
//
// Within one time slice the vertex exponentials are diagonal similarity
// transforms, so G_ii is unchanged by them and the Sherman-Morrison update
// G <- G - x_i G(:,i) (e_i - G(i,:)) has the same form in the frame of the
// slice-start matrix G0 (the scalings are applied at the end of the slice by
// the hopping GEMMs).  Accepting flips at sites S with Delta_S turns G0 into
//   G = G0 - G0(:,S) Delta_S Gamma^-1 (E_S - G0(S,:)),
//   Gamma = 1 + (1 - G0(S,S)) Delta_S,
// and the ratio for a new site j is the Schur complement
//   1 + Delta_j (1 - G0_jj - G0(j,S) Delta_S Gamma^-1 G0(S,j)),
// exactly Upgrade2's Mat(1,1) for the current G.  A block of nq consecutive
// visits therefore needs only G0(Sblk, Sblk) (staged in shared memory) and the
// bordered inverse Gamma^-1 (m <= nq); the O(N^2) work is one rank-m GEMM flush.
#pragma once
#include "common.cuh"

#define UPD_KMAX 32
#define UPD_SMEM_BYTES (4 * UPD_KMAX * (UPD_KMAX + 1) * 16)

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
  int dir;        // 0: up pass (n = q), 1: down pass (n = M-1-q)
  int q0, nq;     // visit positions q0 .. q0+nq-1 of this slice
  int visit_base; // visit index (within the sweep) of position 0 of this slice
  zd* G; long long sG;  // [chain][F][N][N]
  VertexDev V;
  int8_t* fields;       // [chain][L][M]
  const double* draws; long long sDraws;  // [chain][6*M*L] or null
  const unsigned long long* rngkey;      // [chain]
  const unsigned long long* rngctr;      // [chain] counter of draw 0 of this sweep
  zd* phase;            // [chain]
  int* m_out;           // [chain]
  int* sites_out;       // [chain][UPD_KMAX]
  zd* W_out;            // [chain][F][UPD_KMAX][UPD_KMAX], W = Delta_S Gamma^-1 (row-major l,l')
  long long* cnt;       // [chain][4] n_prop, n_acc, n_prop_eff, n_acc_eff
  int8_t* rec_acc; zd* rec_ratio; long long sRec;
  FieldTables ft;
};

ALF_DEV int nranf3(double r) {
  // nint(r*3 + 0.5) clamped to [1,3] (random_wrap_mod.F90:159-168); no contraction.
  double y = __dadd_rn(__dmul_rn(r, 3.0), 0.5);
  int v = (int)round(y);
  return v < 1 ? 1 : (v > 3 ? 3 : v);
}

// One CTA per chain, 64 threads: warp f handles flavour f.
__global__ void __launch_bounds__(64) k_update_block(UpdParams p) {
  const int c = blockIdx.x;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int N = p.N, F = p.F, M = p.M, nq = p.nq;
  extern __shared__ zd upd_smem[];
  // G0(site_a, site_b) as Gs[f][a][b] and Gamma^-1 as Gi[f][l][l'] (dynamic shared memory)
  zd (*Gs)[UPD_KMAX][UPD_KMAX + 1] = reinterpret_cast<zd (*)[UPD_KMAX][UPD_KMAX + 1]>(upd_smem);
  zd (*Gi)[UPD_KMAX][UPD_KMAX + 1] =
      reinterpret_cast<zd (*)[UPD_KMAX][UPD_KMAX + 1]>(upd_smem + 2 * UPD_KMAX * (UPD_KMAX + 1));
  __shared__ zd Dl[2][UPD_KMAX];                 // Delta of accepted (by accept order)
  __shared__ int Sq[UPD_KMAX];                    // block position of accepted, by accept order
  __shared__ int sites[UPD_KMAX];                 // site of block position
  __shared__ int vtx[UPD_KMAX];                   // vertex n of block position
  __shared__ zd yv[2][UPD_KMAX];
  __shared__ zd v_g[2][UPD_KMAX], v_al[2][UPD_KMAX];
  __shared__ double v_E[2][UPD_KMAX];
  __shared__ int v_s[UPD_KMAX], v_t[UPD_KMAX];
  __shared__ double v_u[UPD_KMAX][3];
  __shared__ zd Dcand[2], Rf[2], delta_new[2];
  __shared__ int s_m, s_acc, s_snew;
  __shared__ zd s_phase;

  zd* G = p.G + (long long)c * p.sG;
  const int* site = p.V.site + (long long)c * p.V.sK;
  const zd* gg = p.V.g + (long long)c * p.V.sK;
  const zd* al = p.V.alpha + (long long)c * p.V.sK;
  const double* EE = p.V.E + (long long)c * p.V.sK;
  const int8_t* ty = p.V.type + (long long)c * p.V.sK;
  int8_t* fl = p.fields + (long long)c * p.L * M + (long long)(p.nt1 - 1) * M;

  for (int q = threadIdx.x; q < nq; q += blockDim.x) {
    int pos = p.q0 + q;
    int n = p.dir == 0 ? pos : M - 1 - pos;
    vtx[q] = n;
    sites[q] = site[n];  // flavour 0 site; single-site diagonal vertices share P across flavours
    v_s[q] = fl[n];
    v_t[q] = ty[n];
    for (int f = 0; f < F; ++f) {
      v_g[f][q] = gg[f * M + n];
      v_al[f][q] = al[f * M + n];
      v_E[f][q] = EE[f * M + n];
    }
    const int v = p.visit_base + pos;
    if (p.draws) {
      const double* d = p.draws + (long long)c * p.sDraws + 3ll * v;
      v_u[q][0] = d[0]; v_u[q][1] = d[1]; v_u[q][2] = d[2];
    } else {
      unsigned long long key = p.rngkey[c], ctr = p.rngctr[c] + 3ull * v;
      v_u[q][0] = alf_uniform(key, ctr); v_u[q][1] = alf_uniform(key, ctr + 1); v_u[q][2] = alf_uniform(key, ctr + 2);
    }
  }
  if (threadIdx.x == 0) { s_m = 0; s_phase = p.phase[c]; }
  __syncthreads();
  // Stage G0(Sblk, Sblk) for each flavour.
  for (int e = threadIdx.x; e < F * nq * nq; e += blockDim.x) {
    int f = e / (nq * nq), r = e % (nq * nq);
    int a = r % nq, b = r / nq;
    Gs[f][a][b] = G[(long long)f * N * N + sites[a] + (long long)sites[b] * N];
  }
  __syncthreads();

  long long n_prop = 0, n_acc = 0;
  for (int q = 0; q < nq; ++q) {
    const int n = vtx[q];
    const int v = p.visit_base + p.q0 + q;
    const int m = s_m;
    const double u0 = v_u[q][0], u1 = v_u[q][1], u2 = v_u[q][2];
    const int s_old = v_s[q];
    const int tp = v_t[q];
    const int s_new = (tp == 1) ? -s_old : (int)p.ft.flip[s_old + 2][nranf3(u0) - 1];
    const bool propose = 1.5 > u1;  // T0_proposal (Wrapgr_mod.F90:123,133); always true
    if (w < F) {
      const int f = w;
      const double dphi = p.ft.phi[tp - 1][s_new + 2] - p.ft.phi[tp - 1][s_old + 2];
      const zd Z1 = zscale(v_g[f][q], dphi);
      const zd myexp = zexp(zscale(Z1, v_E[f][q]));
      const zd Dj = zsub(myexp, zmk(1.0, 0.0));
      // y = Gamma^-1 g, g_l = G0(s_l, j)
      zd corr_l = zmk(0.0, 0.0);
      if (lane < m) {
        zd y = zmk(0.0, 0.0);
        for (int l2 = 0; l2 < m; ++l2) y = zadd(y, zmul(Gi[f][lane][l2], Gs[f][Sq[l2]][q]));
        yv[f][lane] = y;
        corr_l = zmul(zmul(Gs[f][q][Sq[lane]], Dl[f][lane]), y);
      }
      zd corr = warp_zsum(corr_l);
      if (lane == 0) {
        zd gcur = zadd(Gs[f][q][q], corr);
        zd mat = zadd(myexp, zneg(zmul(Dj, gcur)));  // Mat(1,1) = myexp - Z*G(P,P)
        Dcand[f] = mat;
        Rf[f] = zmul(mat, zexp(zmul(Z1, v_al[f][q])));
        delta_new[f] = Dj;
      }
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      int acc = 0;
      zd R = zmk(0.0, 0.0);
      if (propose) {
        R = Rf[0];
        for (int f = 1; f < F; ++f) R = zmul(R, Rf[f]);
        zd Rp = R;
        for (int e = 1; e < p.NSUN; ++e) Rp = zmul(Rp, R);
        R = zscale(Rp, p.ft.gama[tp - 1][s_new + 2] / p.ft.gama[tp - 1][s_old + 2]);
        zd ph = s_phase;
        double weight = fabs(zmul(ph, R).x / ph.x);
        acc = weight > u2;
        if (acc) {
          double ar = sqrt(zmul(R, zconj(R)).x);
          zd pr = zmul(ph, R);
          s_phase = zmk(pr.x / ar, pr.y / ar);
        }
      }
      if (p.rec_acc) {
        p.rec_acc[(long long)c * p.sRec + v] = (int8_t)acc;
        p.rec_ratio[(long long)c * p.sRec + v] = R;
      }
      s_acc = acc;
      s_snew = s_new;
    }
    __syncthreads();
    n_prop += propose ? 1 : 0;
    if (s_acc) {
      n_acc += 1;
      if (w < F) {
        const int f = w;
        const zd sinv = zinv(Dcand[f]);
        const zd Dj = delta_new[f];
        // z_l' = sum_l G0(j, s_l) Delta_l Gi[l][l']
        zd z = zmk(0.0, 0.0);
        if (lane < m) {
          for (int l = 0; l < m; ++l) z = zadd(z, zmul(zmul(Gs[f][q][Sq[l]], Dl[f][l]), Gi[f][l][lane]));
        }
        __syncwarp();
        if (lane < m) {
          // column lane of the bordered inverse
          const zd zs = zmul(z, sinv);
          for (int l = 0; l < m; ++l) Gi[f][l][lane] = zadd(Gi[f][l][lane], zmul(zmul(Dj, yv[f][l]), zs));
          Gi[f][m][lane] = zs;
          Gi[f][lane][m] = zmul(zmul(Dj, yv[f][lane]), sinv);
        }
        if (lane == 0) {
          Gi[f][m][m] = sinv;
          Dl[f][m] = Dj;
        }
      }
      if (threadIdx.x == 0) {
        Sq[m] = q;
        s_m = m + 1;
        fl[n] = (int8_t)s_snew;
      }
    }
    __syncthreads();
  }
  // Outputs for the flush: sites and W = Delta_S Gamma^-1.
  const int m = s_m;
  for (int e = threadIdx.x; e < F * m * m; e += blockDim.x) {
    int f = e / (m * m), r = e % (m * m), l = r / m, l2 = r % m;
    p.W_out[(((long long)c * 2 + f) * UPD_KMAX + l) * UPD_KMAX + l2] = zmul(Dl[f][l], Gi[f][l][l2]);
  }
  for (int l = threadIdx.x; l < m; l += blockDim.x) p.sites_out[(long long)c * UPD_KMAX + l] = sites[Sq[l]];
  if (threadIdx.x == 0) {
    p.m_out[c] = m;
    p.phase[c] = s_phase;
    long long* cn = p.cnt + 4ll * c;
    cn[0] += n_prop; cn[1] += n_acc; cn[2] += nq; cn[3] += n_acc;
  }
}

// Flush operands, spread over the GPU:
//   X(:, l) = G0(:, s_l)                           (k_flush_x: one thread per (row, l))
//   Y(l, :) = sum_l' W(l,l') (e_{s_l'} - G0(s_l', :))  (k_flush_y: one thread per (l, column))
// X: [chain][2][N][KMAX] col-major (ld N); Y: [chain][2][KMAX][N] col-major (ld KMAX).
__global__ void k_flush_x(const zd* G, long long sG, int N, int F, const int* m_in, const int* sites, zd* X) {
  const int b = blockIdx.y, c = b / F, f = b % F;
  const int m = m_in[c];
  const long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (e >= (long long)N * m) return;
  const int row = e % N, l = e / N;
  const int s = sites[(long long)c * UPD_KMAX + l];
  X[((long long)c * 2 + f) * N * UPD_KMAX + row + (long long)l * N] =
      G[(long long)c * sG + (long long)f * N * N + row + (long long)s * N];
}

// block: 32 x 8 threads = (l, column); grid (ceil(N/8), B)
__global__ void k_flush_y(const zd* G, long long sG, int N, int F, const int* m_in, const int* sites, const zd* W,
                          zd* Y) {
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
  const zd* Gf = G + (long long)c * sG + (long long)f * N * N;
  if (col < N && tx < m) {
    const int s = st[tx];
    zd gv = Gf[s + (long long)col * N];
    gb[ty][tx] = zsub(zmk(s == col ? 1.0 : 0.0, 0.0), gv);
  }
  __syncthreads();
  if (col < N && tx < m) {
    zd y = zmk(0.0, 0.0);
    for (int l2 = 0; l2 < m; ++l2) y = zadd(y, zmul(Ws[tx][l2], gb[ty][l2]));
    Y[((long long)c * 2 + f) * N * UPD_KMAX + tx + (long long)col * UPD_KMAX] = y;
  }
}
