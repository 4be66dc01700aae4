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
// applied by one rank-m GEMM flush; W = Delta_S Gamma^-1 is formed at block
// end by the same kernel.
//
// G is complex128 in both precision forms.  The sequential chain (ratios,
// Metropolis test, phase), the Ghat rank-1 updates and Gamma^-1 run in FP64
// (plain form) or double-float (mixed form, dfloat.cuh, ~2^-46 relative
// rounding).  GB300's FP64 dependent latency (63-76 cycles, ~560 for a
// division) sets the cost of every visit, so the chain avoids divisions and
// square roots: the Metropolis test is division-free, the reciprocal is a
// Newton iteration, and the phase stays unnormalised until the block ends.
#pragma once
#include "common.cuh"
#include "arith.cuh"

#define UPD_KMAX 32
#define UPD_THREADS 256

struct VertexDev {
  // per chain: K = F*M entries, index k = nf*M + n
  const int* site;       // P(1), 0-based
  const int8_t* type;    // 1 or 2
  long long sK;          // per-chain stride in entries (F*M)
};
struct UpdTab;

struct UpdParams {
  int N, F, M, L, NSUN;
  int nt1;        // slice, 1-based
  int dir;        // 0: up pass (n = pos), 1: down pass (n = M-1-pos)
  int q0, nq;     // visit positions q0 .. q0+nq-1 of this slice
  int visit_base; // visit index (within the sweep) of position 0 of this slice
  int nChains;
  const void* G; long long sG;  // [chain][F][N][N] complex128
  VertexDev V;
  const UpdTab* tab;    // [chain][F*M][5][3]
  int8_t* fields;       // [chain][L][M]
  const double* draws; long long sDraws;  // [chain][6*M*L] or null
  const unsigned long long* rngkey;      // [chain]
  const unsigned long long* rngctr;      // [chain] counter of draw 0 of this sweep
  zd* phase;            // [chain]
  int* m_out;           // [chain], then [chain][F] (per-GEMM-batch rank)
  zd* W;                // [chain][2][UPD_KMAX][UPD_KMAX]  Delta_S Gamma^-1
  int* sites_out;       // [chain][UPD_KMAX]  accepted sites, accept order
  zd* delta_out;        // [chain][2][UPD_KMAX] Delta of accepted sites
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

// Per-visit transition data, precomputed per (vertex k, old field s, flip choice):
//   myexp = exp(Z E), dlt = myexp - 1, expal = exp(Z alpha),  Z = g (phi(s_new) - phi(s_old))
// (Upgrade2's Mat(1,1) = myexp - dlt G(P,P), Hamiltonian_main_mod.F90 ratio factors).
struct UpdTab {
  zd myexp, dlt, expal;
};

// One CTA of UPD_THREADS threads per chain.  Dynamic shared memory:
//   Gh[F][KMAX][KMAX+1]  the block Ghat, updated in place (arithmetic A)
//   G0[F][KMAX][KMAX+1]  Ghat at block entry; reused as the ping-pong buffer of the
//                        Gauss-Jordan inversion of Gamma.
// Warp 0 runs the sequential Metropolis chain (all lanes compute the same scalars;
// lane a handles row a of a column).  While warps 1..7 apply the rank-1 update of
// an accepted visit q to rows a > q and columns b > q+1, warp 0 updates column q+1
// itself and already decides visit q+1 from its new diagonal: one block barrier
// per visit.  At block end, W = Delta_S Gamma^-1 is formed by Gauss-Jordan
// elimination without pivoting: the pivots in accept order are the accepted
// visits' own 1 + Delta (1 - G_jj) factors (the Sherman-Morrison sequence is the LU
// factorisation of Gamma in that order), non-zero because a zero factor gives
// weight 0 and is rejected.
template <class A>
__global__ void __launch_bounds__(UPD_THREADS) k_update(UpdParams p) {
  typedef typename A::Z Z;
  typedef typename A::R R;
  constexpr int KM = UPD_KMAX, LD = UPD_KMAX + 1, NW = UPD_THREADS / 32;
  const int c = blockIdx.x, tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int N = p.N, F = p.F, M = p.M, nq = p.nq;
  extern __shared__ __align__(16) unsigned char upd_raw[];
  Z* Gh = reinterpret_cast<Z*>(upd_raw);
  Z* G0 = Gh + 2 * KM * LD;
  __shared__ Z s_mye[2][KM], s_dlt[2][KM], s_tcol[2][2][KM], s_K[KM], s_rowt[2][KM], s_piv[2][2];
  __shared__ zd s_dlt64[2][KM];
  __shared__ R s_u2[KM], s_gr[KM];
  __shared__ int s_site[KM], s_vtx[KM], s_snew[KM], s_prop[KM], s_accq[KM], s_acc[2];
  __shared__ short s_ij[KM * KM];
  __shared__ int s_m;

  const double2* G = reinterpret_cast<const double2*>(p.G) + (long long)c * p.sG;
  const int* site = p.V.site + (long long)c * p.V.sK;
  const int8_t* ty = p.V.type + (long long)c * p.V.sK;
  const UpdTab* tab = p.tab + (long long)c * p.V.sK * 15;
  int8_t* fl = p.fields + (long long)c * p.L * M + (long long)(p.nt1 - 1) * M;
  const long long NN = (long long)N * N;

  // Prologue: each vertex is visited once per block, so its old field is the field at
  // block start and every visit's proposal, draws and transition factors are known.
  if (tid < nq) {
    const int q = tid, pos = p.q0 + q;
    const int n = p.dir == 0 ? pos : M - 1 - pos;
    s_vtx[q] = n;
    s_site[q] = site[n];
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
    const int ch = (tp == 1) ? 0 : nranf3(u0) - 1;
    const int sn = (tp == 1) ? -so : (int)p.ft.flip[so + 2][ch];
    s_snew[q] = sn;
    s_prop[q] = 1.5 > u1;  // T0_proposal (Wrapgr_mod.F90:123,133); always true
    s_u2[q] = A::mkr(uu2);
    s_gr[q] = A::mkr(p.ft.grat[tp - 1][so + 2][sn + 2]);
    zd K = zmk(1.0, 0.0);
    for (int f = 0; f < F; ++f) {
      const UpdTab e = tab[((long long)(f * M + n) * 5 + so + 2) * 3 + ch];
      s_mye[f][q] = A::mk(e.myexp);
      s_dlt[f][q] = A::mk(e.dlt);
      s_dlt64[f][q] = e.dlt;
      K = (f == 0) ? e.expal : zmul(K, e.expal);
    }
    s_K[q] = A::mk(K);
  }
  __syncthreads();
  for (int a = warp; a < nq; a += NW)
    if (lane < nq)
      for (int f = 0; f < F; ++f) {
        const Z v = A::mk(G[f * NN + s_site[a] + (long long)s_site[lane] * N]);
        Gh[(f * KM + a) * LD + lane] = v;
        G0[(f * KM + a) * LD + lane] = v;
      }
  __syncthreads();

  // warp-0 state (identical in all lanes)
  Z ph = A::mk(p.phase[c]);  // kept unnormalised (only its direction enters the weight)
  int m = 0;
  long long n_prop = 0;
  // Decide visit v from the current Ghat(v,v) (gd) and column Ghat(lane, v) (gc, lanes > v).
  auto decide = [&](int v, const Z* gd, const Z* gc) {
    int acc = 0;
    Z Rt = A::zero();
    if (s_prop[v]) {
      Z D[2];
#pragma unroll
      for (int f = 0; f < 2; ++f)  // Mat(1,1) = myexp - Delta G(P,P)
        if (f < F) D[f] = A::sub(s_mye[f][v], A::mul(s_dlt[f][v], gd[f]));
      Rt = (F == 2) ? A::mul(D[0], D[1]) : D[0];
      Rt = A::mul(Rt, s_K[v]);
      Z Rp = Rt;
      for (int e = 1; e < p.NSUN; ++e) Rp = A::mul(Rp, Rt);
      Rt = A::scale(Rp, s_gr[v]);
      // weight = |Re(phase R) / Re(phase)| > u  (Wrapgr_mod.F90:141-143), division-free
      const R num = A::absr(A::re_mul(ph, Rt));
      const R den = A::mulr(A::absr(A::re(ph)), s_u2[v]);
      acc = A::gt(num, den);
      if (acc) {
        ph = A::renorm(A::mul(ph, Rt));
#pragma unroll
        for (int f = 0; f < 2; ++f)
          if (f < F) {
            const Z x = A::mul(s_dlt[f][v], A::rcp(D[f]));  // Delta / Mat(1,1)
            if (lane > v && lane < nq) s_tcol[v & 1][f][lane] = A::mul(x, gc[f]);
          }
      }
    }
    n_prop += s_prop[v];
    if (lane == 0) {
      if (p.rec_acc) {
        const long long r = (long long)c * p.sRec + p.visit_base + p.q0 + v;
        p.rec_acc[r] = (int8_t)acc;
        p.rec_ratio[r] = A::wide(Rt);
      }
      if (acc) {
        s_accq[m] = v;
        p.sites_out[(long long)c * KM + m] = s_site[v];
        for (int f = 0; f < F; ++f) p.delta_out[((long long)c * 2 + f) * KM + m] = s_dlt64[f][v];
        fl[s_vtx[v]] = (int8_t)s_snew[v];
      }
      s_acc[v & 1] = acc;
    }
    m += acc;
  };

  if (warp == 0) {
    Z gd[2], gc[2];
#pragma unroll
    for (int f = 0; f < 2; ++f)
      if (f < F) {
        gc[f] = (lane < nq) ? Gh[(f * KM + lane) * LD] : A::zero();
        gd[f] = Gh[f * KM * LD];
      }
    decide(0, gd, gc);
  }
  __syncthreads();
  for (int q = 0; q < nq; ++q) {
    const int acc = s_acc[q & 1];
    if (warp == 0) {
      if (q + 1 < nq) {
        const int v = q + 1;
        Z gd[2], gc[2];
#pragma unroll
        for (int f = 0; f < 2; ++f)
          if (f < F) {
            Z col = (lane < nq) ? Gh[(f * KM + lane) * LD + v] : A::zero();
            if (acc && lane > q && lane < nq) {  // column v of the rank-1 update of visit q
              col = A::mac(col, s_tcol[q & 1][f][lane], Gh[(f * KM + q) * LD + v]);
              Gh[(f * KM + lane) * LD + v] = col;
            }
            gc[f] = col;
            gd[f] = A::shfl(col, v);
          }
        decide(v, gd, gc);
      }
    } else if (acc) {
      // Ghat(a,b) += x Ghat(a,q) Ghat(q,b), rows a > q, columns b > q+1
      const int b = lane;
      if (b > q + 1 && b < nq)
        for (int f = 0; f < F; ++f)
          for (int a = q + warp; a < nq; a += NW - 1) {
            Z* g = Gh + (f * KM + a) * LD + b;
            *g = A::mac(*g, s_tcol[q & 1][f][a], Gh[(f * KM + q) * LD + b]);
          }
    }
    __syncthreads();
  }
  if (tid == 0) s_m = m;
  __syncthreads();
  m = s_m;
  if (m > 0) {
    const int FMM = F * m * m;
    for (int e = tid; e < m * m; e += UPD_THREADS) s_ij[e] = (short)(((e / m) << 6) | (e % m));
    // Gamma(l,l') = delta_ll' + (delta_ll' - G0(s_l, s_l')) Delta_l'  in Gh (accept order)
    for (int l = warp; l < m; l += NW)
      if (lane < m)
        for (int f = 0; f < F; ++f) {
          const int l2 = lane;
          const Z g = G0[(f * KM + s_accq[l]) * LD + s_accq[l2]];
          Z v = A::mul(A::sub(l == l2 ? A::one() : A::zero(), g), s_dlt[f][s_accq[l2]]);
          if (l == l2) v = A::add(v, A::one());
          Gh[(f * KM + l) * LD + l2] = v;
        }
    __syncthreads();
    if (tid < F) s_piv[0][tid] = A::rcp(Gh[(tid * KM) * LD]);
    // in-place Gauss-Jordan inversion, ping-pong between Gh and G0
    Z* Ga = Gh;
    Z* Gb = G0;
    for (int k = 0; k < m; ++k) {
      __syncthreads();
      if (warp < F && lane < m) s_rowt[warp][lane] = A::mul(Ga[(warp * KM + lane) * LD + k], s_piv[k & 1][warp]);
      __syncthreads();
      for (int e = tid; e < FMM; e += UPD_THREADS) {
        const int f = e >= m * m, r = e - f * m * m;
        const int i = s_ij[r] >> 6, j = s_ij[r] & 63;
        const Z pinv = s_piv[k & 1][f];
        Z v;
        if (i == k && j == k) v = pinv;
        else if (i == k) v = A::mul(Ga[(f * KM + k) * LD + j], pinv);
        else if (j == k) v = A::neg(s_rowt[f][i]);
        else v = A::mac(Ga[(f * KM + i) * LD + j], A::neg(s_rowt[f][i]), Ga[(f * KM + k) * LD + j]);
        Gb[(f * KM + i) * LD + j] = v;
        if (i == k + 1 && j == k + 1) s_piv[(k + 1) & 1][f] = A::rcp(v);
      }
      Z* t = Ga; Ga = Gb; Gb = t;
    }
    __syncthreads();
    // W(l, l') = Delta_l Gamma^-1(l, l')
    for (int l = warp; l < m; l += NW)
      if (lane < m)
        for (int f = 0; f < F; ++f)
          p.W[(((long long)c * 2 + f) * KM + l) * KM + lane] =
              zmul(s_dlt64[f][s_accq[l]], A::wide(Ga[(f * KM + l) * LD + lane]));
  }
  if (tid == 0) {
    p.m_out[c] = m;
    for (int f = 0; f < F; ++f) p.m_out[p.nChains + c * F + f] = m;
    if (m > 0) p.phase[c] = A::unit(ph);
    long long* cn = p.cnt + 4ll * c;
    cn[0] += n_prop; cn[1] += m; cn[2] += nq; cn[3] += m;
  }
}

constexpr size_t upd_smem_bytes() { return 2ull * 2 * UPD_KMAX * (UPD_KMAX + 1) * 16; }  // Z is 16 bytes

// Flush operands for G = G0 - X Y (one launch, spread over the GPU):
//   X(:, l) = G0(:, s_l)
//   Y(l, :) = sum_l' W(l,l') (e_{s_l'} - G0(s_l', :))
// block 32 x 8 threads = (l, column / row); grid (ceil(N/8), chains*flavours).
// X: [chain][2][N][KMAX] col-major (ld N); Y: [chain][2][KMAX][N] col-major (ld KMAX).
__global__ void k_flush_xy(const zd* Gv, long long sG, int N, int F, const int* m_in, const int* sites, const zd* W,
                           zd* X, zd* Y) {
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
  const zd* Gf = Gv + (long long)c * sG + (long long)f * N * N;
  const long long xy = ((long long)c * 2 + f) * N * UPD_KMAX;
  if (col < N && tx < m) {
    const int s = st[tx];
    X[xy + col + (long long)tx * N] = Gf[col + (long long)s * N];  // row `col` of X
    gb[ty][tx] = zsub(zmk(s == col ? 1.0 : 0.0, 0.0), Gf[s + (long long)col * N]);
  }
  __syncthreads();
  if (col < N && tx < m) {
    zd y = zmk(0.0, 0.0);
    for (int l2 = 0; l2 < m; ++l2) y = zadd(y, zmul(Ws[tx][l2], gb[ty][l2]));
    Y[xy + tx + (long long)col * UPD_KMAX] = y;
  }
}

