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
// G is complex128 in both precision forms.  The per-flavour determinants
// Mat(1,1) (or the 2x2 determinant of a two-site vertex), the Ghat rank-1 updates
// and Gamma^-1 run in FP64 (plain form) or double-float (mixed form, dfloat.cuh,
// ~2^-46 relative rounding).  The accumulation of the Metropolis ratio (the
// product over flavours, exp(Z1 alpha), the N_SUN power and the gamma ratio), the
// weight test and the phase are FP64 in both forms.  GB300's FP64 dependent
// latency (63-76 cycles, ~560 for a division) sets the cost of every visit, so
// the chain avoids divisions and square roots: the Metropolis test is
// division-free, the reciprocal is a Newton iteration, and the phase stays
// unnormalised until the block ends.
#pragma once
#include "common.cuh"
#include "arith.cuh"

#define UPD_KMAX 32
#define UPD_THREADS 256

struct VertexDev {
  // per chain: K = F*M entries, index k = nf*M + n
  const int* site;       // site of eigen-index 0 (P(1), 0-based)
  const int* site2;      // site of eigen-index 1, or -1
  const int8_t* nsite;   // positions of the vertex: its non-zero eigenvalues (1 or 2)
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
  // vector vertices (a single-site vertex on a site of a rotated pair: in the rotated basis its
  // one position is the real unit vector u = c_a e_a + c_b e_b); null when the model has none
  const int* vsite2;    // [chain][F*M] site b of a vector vertex, -1 otherwise
  const double* vcoef;  // [chain][F*M][2] (c_a, c_b)
  int* sites2_out;      // [chain][UPD_KMAX] accepted positions: site b or -1
  double* coef_out;     // [chain][UPD_KMAX][2]
  // optional: the block submatrix Ghat = G(P, P) over this block's positions P, staged by
  // k_sub_stage while the previous block's flush still runs ([chain][F][KMAX][KMAX], row a =
  // position a); null: read from G
  const zd* Gsub;
};

// Positions of the block of visits q0 .. q0 + nq - 1 (slice order dir) of chain c: the site of
// every non-zero eigenvalue, in the order k_update numbers them (exclusive prefix sum of the
// vertex sizes over the visits).  Warp-level: every lane of the calling warp takes part;
// returns the position count, writes pos[0 .. np).
ALF_DEV int block_positions(const VertexDev& V, int c, int M, int dir, int q0, int nq, int* pos) {
  const int lane = threadIdx.x & 31;
  const int* site = V.site + (long long)c * V.sK;
  const int* site2 = V.site2 + (long long)c * V.sK;
  const int8_t* nsite = V.nsite + (long long)c * V.sK;
  int w = 0, n = 0;
  if (lane < nq) {
    n = dir == 0 ? q0 + lane : M - 1 - (q0 + lane);
    w = nsite[n];
  }
  int incl = w;
  for (int o = 1; o < 32; o <<= 1) {
    const int t = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += t;
  }
  const int p0 = incl - w;
  for (int I = 0; I < w; ++I) pos[p0 + I] = I ? site2[n] : site[n];
  return __shfl_sync(0xffffffffu, incl, 31);
}

// Snapshot of G over the positions of the next block, taken before the current block's flush
// writes G: Gsnap[chain][f][a][l] = G(P_a, P_l).  Also stores the positions (pos[chain][KMAX],
// npos[chain]).  grid (chains * F), 256 threads.
__global__ void k_sub_gather(const zd* G, long long sG, int N, int F, int M, VertexDev V, int dir, int q0, int nq,
                             zd* Gsnap, int* pos, int* npos) {
  const int b = blockIdx.x, c = b / F, f = b % F, tid = threadIdx.x;
  __shared__ int sp[UPD_KMAX];
  __shared__ int snp;
  if (tid < 32) {
    const int np = block_positions(V, c, M, dir, q0, nq, sp);
    if (tid == 0) snp = np;
  }
  __syncthreads();
  const int np = snp;
  if (f == 0) {
    for (int a = tid; a < np; a += 256) pos[(long long)c * UPD_KMAX + a] = sp[a];
    if (tid == 0) npos[c] = np;
  }
  const zd* Gf = G + (long long)c * sG + (long long)f * N * N;
  zd* out = Gsnap + (long long)b * UPD_KMAX * UPD_KMAX;
  for (int e = tid; e < np * np; e += 256) {
    const int a = e / np, l = e % np;
    out[a * UPD_KMAX + l] = Gf[sp[a] + (long long)sp[l] * N];
  }
}

// The next block's submatrix after the current block's accepted updates, from the snapshot
// and the flush operands: Gsub(a, l) = Gsnap(a, l) - sum_k X(P_a, k) Y(k, P_l), k < m (the same
// Woodbury form the flush applies to all of G).
// grid (ceil(KMAX / 8), chains * F), block (32, 8): (l, a).
template <class A>
__global__ void k_sub_stage(const zd* Gsnap, const int* pos, const int* npos, const int* m_in, int N, int F,
                            const zd* X, const zd* Y, zd* Gsub) {
  typedef typename A::Z Z;
  const int b = blockIdx.y, c = b / F, f = b % F;
  const int l = threadIdx.x, a = blockIdx.x * 8 + threadIdx.y;
  const int np = npos[c], m = m_in[c];
  if (a >= np || l >= np) return;
  const long long o = (long long)b * UPD_KMAX * UPD_KMAX + a * UPD_KMAX + l;
  const int pa = pos[(long long)c * UPD_KMAX + a], pl = pos[(long long)c * UPD_KMAX + l];
  const long long xy = ((long long)c * 2 + f) * N * UPD_KMAX;
  Z acc = A::zero();
  for (int k = 0; k < m; ++k) acc = A::mac(acc, A::mk(X[xy + pa + (long long)k * N]), A::mk(Y[xy + k + (long long)pl * UPD_KMAX]));
  Gsub[o] = A::wide(A::sub(A::mk(Gsnap[o]), acc));
}

ALF_DEV int nranf3(double r) {
  // nint(r*3 + 0.5) clamped to [1,3] (random_wrap_mod.F90:159-168); no contraction.
  double y = __dadd_rn(__dmul_rn(r, 3.0), 0.5);
  int v = (int)round(y);
  return v < 1 ? 1 : (v > 3 ? 3 : v);
}

// Per-visit transition data, precomputed per (vertex k, old field s, flip choice):
//   myexp_I = exp(Z E_I), dlt_I = myexp_I - 1, expal = exp(Z alpha),  Z = g (phi(s_new) - phi(s_old))
// for the eigen-indices I = 0, 1 (Upgrade2's Mat(I,I) = myexp_I - dlt_I G(P_I,P_I),
// upgrade_mod.F90:140-190).
struct UpdTab {
  zd myexp[2], dlt[2], expal;
};

// One CTA of UPD_THREADS threads per chain.  Dynamic shared memory:
//   Gh[F][KMAX][KMAX+1]  the block Ghat over the block's positions, updated in place
//   G0[F][KMAX][KMAX+1]  Ghat at block entry; reused as the ping-pong buffer of the
//                        Gauss-Jordan inversion of Gamma.
// A position is one non-zero eigenvalue of a vertex (its site in the diagonal basis);
// single-site vertices have one, two-site vertices two consecutive positions whose
// joint ratio is Upgrade2's 2x2 determinant, computed as D_a (1 + Delta_b (1 - G'_bb))
// with G' after the tentative Sherman-Morrison update of position a; an accepted
// two-site vertex is applied as two rank-1 updates, the second decided with the first.
// Warp 0 runs the sequential Metropolis chain (all lanes compute the same scalars;
// lane a handles row a of a column).  While warps 1..7 apply the rank-1 update of an
// accepted position q to rows a > q and the columns beyond those warp 0 needs next,
// warp 0 updates the next one or two columns itself and already decides the next
// position from them: one block barrier per position.  At block end, W = Delta_S Gamma^-1
// is formed by Gauss-Jordan elimination without pivoting: the pivots in accept order
// are the accepted positions' own 1 + Delta (1 - G_jj) factors (the Sherman-Morrison
// sequence is the LU factorisation of Gamma in that order), non-zero because a zero
// factor gives weight 0 and is rejected.
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
  // per position
  __shared__ Z s_mye[2][KM], s_dlt[2][KM], s_tcol[2][2][KM], s_rowt[2][KM], s_piv[2][2];
  __shared__ zd s_dlt64[2][KM];
  __shared__ int s_psite[KM], s_pvis[KM], s_pkind[KM], s_accq[KM], s_acc[2];
  __shared__ int s_psite2[KM];      // vector positions: site b, else -1
  __shared__ double s_pc[KM][2];    // vector positions: (c_a, c_b)
  // per visit (FP64 in both forms: the ratio accumulation)
  __shared__ zd s_K[KM];
  __shared__ double s_u2[KM], s_gr[KM];
  __shared__ int s_vtx[KM], s_snew[KM], s_prop[KM];
  __shared__ short s_ij[KM * KM];
  __shared__ int s_m, s_np;

  const double2* G = reinterpret_cast<const double2*>(p.G) + (long long)c * p.sG;
  const int* site = p.V.site + (long long)c * p.V.sK;
  const int* site2 = p.V.site2 + (long long)c * p.V.sK;
  const int8_t* nsite = p.V.nsite + (long long)c * p.V.sK;
  const int8_t* ty = p.V.type + (long long)c * p.V.sK;
  const UpdTab* tab = p.tab + (long long)c * p.V.sK * 15;
  int8_t* fl = p.fields + (long long)c * p.L * M + (long long)(p.nt1 - 1) * M;
  const long long NN = (long long)N * N;

  // Prologue (warp 0, lane q = visit): each vertex is visited once per block, so its old
  // field is the field at block start and every visit's proposal, draws and transition
  // factors are known; positions by an exclusive prefix sum of the vertex sizes.
  if (warp == 0) {
    const int q = lane;
    int w = 0, n = 0;
    if (q < nq) {
      const int pos = p.q0 + q;
      n = p.dir == 0 ? pos : M - 1 - pos;
      w = nsite[n];
    }
    int incl = w;
    for (int o = 1; o < 32; o <<= 1) {
      const int t = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += t;
    }
    const int p0 = incl - w;
    if (lane == 31) s_np = incl;
    if (q < nq) {
      s_vtx[q] = n;
      const int v = p.visit_base + p.q0 + q;
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
      s_u2[q] = uu2;
      s_gr[q] = p.ft.grat[tp - 1][so + 2][sn + 2];
      zd K = zmk(1.0, 0.0);
      for (int f = 0; f < F; ++f) {
        const UpdTab e = tab[((long long)(f * M + n) * 5 + so + 2) * 3 + ch];
        for (int I = 0; I < w; ++I) {
          s_mye[f][p0 + I] = A::mk(e.myexp[I]);
          s_dlt[f][p0 + I] = A::mk(e.dlt[I]);
          s_dlt64[f][p0 + I] = e.dlt[I];
        }
        K = (f == 0) ? e.expal : zmul(K, e.expal);
      }
      // [prod_f exp(Z1 alpha)]^N_SUN gamma'/gamma: with N_SUN = 1 the gamma ratio joins K
      if (p.NSUN == 1) K = zscale(K, p.ft.grat[tp - 1][so + 2][sn + 2]);
      s_K[q] = K;
      const int vb = p.vsite2 ? p.vsite2[(long long)c * p.V.sK + n] : -1;
      for (int I = 0; I < w; ++I) {
        s_psite[p0 + I] = I ? site2[n] : site[n];
        s_pvis[p0 + I] = q;
        s_pkind[p0 + I] = (w == 2) ? (I ? 2 : 1) : 0;  // 0 single, 1 first of a pair, 2 second
        s_psite2[p0 + I] = (w == 1) ? vb : -1;
        if (vb >= 0) {
          s_pc[p0 + I][0] = p.vcoef[2 * ((long long)c * p.V.sK + n)];
          s_pc[p0 + I][1] = p.vcoef[2 * ((long long)c * p.V.sK + n) + 1];
        }
      }
    }
  }
  __syncthreads();
  const int np = s_np;
  for (int a = warp; a < np; a += NW)
    if (lane < np)
      for (int f = 0; f < F; ++f) {
        zd g = p.Gsub ? p.Gsub[(((long long)c * F + f) * KM + a) * KM + lane]
                      : G[f * NN + s_psite[a] + (long long)s_psite[lane] * N];
        if (p.vsite2 && (s_psite2[a] >= 0 || s_psite2[lane] >= 0)) {
          // Ghat(a, l) = v_a^T G v_l over the (up to two) sites of each position
          const int ia[2] = {s_psite[a], s_psite2[a]}, il[2] = {s_psite[lane], s_psite2[lane]};
          const double ca[2] = {s_psite2[a] >= 0 ? s_pc[a][0] : 1.0, s_psite2[a] >= 0 ? s_pc[a][1] : 0.0};
          const double cl[2] = {s_psite2[lane] >= 0 ? s_pc[lane][0] : 1.0, s_psite2[lane] >= 0 ? s_pc[lane][1] : 0.0};
          g = zmk(0.0, 0.0);
          for (int x = 0; x < 2; ++x)
            for (int y = 0; y < 2; ++y)
              if (ia[x] >= 0 && il[y] >= 0 && ca[x] != 0.0 && cl[y] != 0.0)
                g = zadd(g, zscale(G[f * NN + ia[x] + (long long)il[y] * N], ca[x] * cl[y]));
        }
        const Z v = A::mk(g);
        Gh[(f * KM + a) * LD + lane] = v;
        G0[(f * KM + a) * LD + lane] = v;
      }
  __syncthreads();

  // warp-0 state (identical in all lanes)
  zd ph = p.phase[c];  // FP64, kept unnormalised within a block (only its direction enters the weight)
  int m = 0, nacc = 0, pend = 0;
  long long n_prop = 0;
  auto accept_pos = [&](int v) {
    if (lane == 0) {
      s_accq[m] = v;
      p.sites_out[(long long)c * KM + m] = s_psite[v];
      if (p.sites2_out) {
        p.sites2_out[(long long)c * KM + m] = s_psite2[v];
        if (s_psite2[v] >= 0) {
          p.coef_out[2 * ((long long)c * KM + m)] = s_pc[v][0];
          p.coef_out[2 * ((long long)c * KM + m) + 1] = s_pc[v][1];
        }
      }
      for (int f = 0; f < F; ++f) p.delta_out[((long long)c * 2 + f) * KM + m] = s_dlt64[f][v];
    }
    m += 1;
  };
  // Decide position v from the current column v (gc, diagonal gd) and, for the first
  // position of a pair, column v+1 (gc2).  Second positions follow their pair's decision.
  auto decide = [&](int v, const Z* gd, const Z* gc, const Z* gc2) {
    const int kind = s_pkind[v];
    int acc = 0;
    const int fo = (F == 2) ? (lane & 1) : 0;  // flavour of this lane's scalar work
    if (kind == 2) {  // second position of an accepted / rejected pair
      acc = pend;
      if (acc) {
        const Z D = A::sub(s_mye[fo][v], A::mul(s_dlt[fo][v], fo ? gd[1] : gd[0]));
        const Z xm = A::mul(s_dlt[fo][v], A::rcp(D));
        const Z x[2] = {A::shfl(xm, 0), A::shfl(xm, 1)};
#pragma unroll
        for (int f = 0; f < 2; ++f)
          if (f < F && lane > v && lane < np) s_tcol[v & 1][f][lane] = A::mul(x[f], gc[f]);
        accept_pos(v);
      }
      if (lane == 0) s_acc[v & 1] = acc;
      return;
    }
    const int q = s_pvis[v];
    zd Rt = zmk(0.0, 0.0);
    if (s_prop[q]) {
      // lane parity carries flavour fo: Mat(1,1) = myexp - Delta G(P,P), and for the first
      // position of a pair the 2x2 determinant D_a (myexp_b - Delta_b G'_bb)
      const Z D = A::sub(s_mye[fo][v], A::mul(s_dlt[fo][v], fo ? gd[1] : gd[0]));
      Z Rm = D, xm = A::zero();
      if (kind == 1) {
        xm = A::mul(s_dlt[fo][v], A::rcp(D));
        const int w = v + 1;
        const Z c2 = fo ? gc2[1] : gc2[0], c1 = fo ? gc[1] : gc[0];
        const Z gww = A::shfl(c2, w), gvw = A::shfl(c2, v), gwv = A::shfl(c1, w);
        const Z gp = A::mac(gww, A::mul(xm, gwv), gvw);
        Rm = A::mul(D, A::sub(s_mye[fo][w], A::mul(s_dlt[fo][w], gp)));
      }
      // the ratio is accumulated in FP64: flavour product, exp(Z1 alpha), N_SUN power
      const zd Rm64 = A::wide(Rm);
      Rt = (F == 2) ? zmul(ArD::shfl(Rm64, 0), ArD::shfl(Rm64, 1)) : Rm64;
      if (p.NSUN == 1) {
        Rt = zmul(Rt, s_K[q]);  // K carries the gamma ratio (prologue)
      } else {
        Rt = zmul(Rt, s_K[q]);
        zd Rp = Rt;
        for (int e = 1; e < p.NSUN; ++e) Rp = zmul(Rp, Rt);
        Rt = zscale(Rp, s_gr[q]);
      }
      // weight = |Re(phase R) / Re(phase)| > u  (Wrapgr_mod.F90:141-143), division-free, FP64
      const double num = fabs(ph.x * Rt.x - ph.y * Rt.y);
      const double den = fabs(ph.x) * s_u2[q];
      acc = num > den;
      if (acc) {
        ph = zmul(ph, Rt);
        if (kind != 1) xm = A::mul(s_dlt[fo][v], A::rcp(D));  // Delta / Mat(1,1)
        const Z x[2] = {A::shfl(xm, 0), A::shfl(xm, 1)};
#pragma unroll
        for (int f = 0; f < 2; ++f)
          if (f < F && lane > v && lane < np) s_tcol[v & 1][f][lane] = A::mul(F == 2 ? x[f] : xm, gc[f]);
      }
    }
    n_prop += s_prop[q];
    if (lane == 0) {
      if (p.rec_acc) {
        const long long r = (long long)c * p.sRec + p.visit_base + p.q0 + q;
        p.rec_acc[r] = (int8_t)acc;
        p.rec_ratio[r] = Rt;
      }
      if (acc) fl[s_vtx[q]] = (int8_t)s_snew[q];
      s_acc[v & 1] = acc;
    }
    if (acc) { accept_pos(v); nacc += 1; }
    pend = acc;
  };

  if (warp == 0) {
    Z gd[2], gc[2], gc2[2];
#pragma unroll
    for (int f = 0; f < 2; ++f)
      if (f < F) {
        gc[f] = (lane < np) ? Gh[(f * KM + lane) * LD] : A::zero();
        gc2[f] = (lane < np && np > 1) ? Gh[(f * KM + lane) * LD + 1] : A::zero();
        gd[f] = Gh[f * KM * LD];
      }
    decide(0, gd, gc, gc2);
  }
  __syncthreads();
  for (int q = 0; q < np; ++q) {
    const int acc = s_acc[q & 1];
    const int v = q + 1;
    // columns warp 0 brings up to date for its next decision: v, and v+1 if v opens a pair
    const int wc = (v < np && s_pkind[v] == 1) ? 2 : 1;
    if (warp == 0) {
      if (v < np) {
        Z gd[2], gc[2], gc2[2];
#pragma unroll
        for (int f = 0; f < 2; ++f)
          if (f < F) {
#pragma unroll
            for (int t = 0; t < 2; ++t) {
              if (t >= wc) continue;
              const int col_i = v + t;
              Z col = (lane < np) ? Gh[(f * KM + lane) * LD + col_i] : A::zero();
              if (acc && lane > q && lane < np) {  // column col_i of the rank-1 update of position q
                col = A::mac(col, s_tcol[q & 1][f][lane], Gh[(f * KM + q) * LD + col_i]);
                Gh[(f * KM + lane) * LD + col_i] = col;
              }
              if (t == 0) gc[f] = col; else gc2[f] = col;
            }
            gd[f] = A::shfl(gc[f], v);
          }
        decide(v, gd, gc, gc2);
      }
    } else if (acc && warp != 4) {
      // Ghat(a,b) += x Ghat(a,q) Ghat(q,b), rows a > q, columns b > q + wc.  Warp 4 shares
      // warp 0's SM sub-partition (FP64 unit) and stays idle so the chain is not delayed.
      const int wk = warp < 4 ? warp : warp - 1;  // 1..6
      const int b = lane;
      if (b > q + wc && b < np)
        for (int f = 0; f < F; ++f)
          for (int a = q + wk; a < np; a += NW - 2) {
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
    if (m > 0) p.phase[c] = ArD::unit(ph);
    long long* cn = p.cnt + 4ll * c;
    cn[0] += n_prop; cn[1] += nacc; cn[2] += nq; cn[3] += nacc;
  }
}

constexpr size_t upd_smem_bytes() { return 2ull * 2 * UPD_KMAX * (UPD_KMAX + 1) * 16; }  // Z is 16 bytes

// Flush operands for G = G0 - X Y (one launch, spread over the GPU; the m x m x N product of
// Y in the precision form's arithmetic, double-float in the mixed form):
//   X(:, l) = G0 v_l
//   Y(l, :) = sum_l' W(l,l') (v_l'^T - v_l'^T G0)
// with v_l = e_{s_l}, or c_a e_a + c_b e_b for a vector position (sites2 / coefs, may be null).
// block 32 x 8 threads = (l, column / row); grid (ceil(N/8), chains*flavours).
// X: [chain][2][N][KMAX] col-major (ld N); Y: [chain][2][KMAX][N] col-major (ld KMAX).
template <class A>
__global__ void k_flush_xy(const zd* Gv, long long sG, int N, int F, const int* m_in, const int* sites, const zd* W,
                           zd* X, zd* Y, const int* sites2 = nullptr, const double* coefs = nullptr) {
  typedef typename A::Z Z;
  const int b = blockIdx.y, c = b / F, f = b % F;
  const int m = m_in[c];
  if (m == 0) return;
  __shared__ Z Ws[UPD_KMAX][UPD_KMAX + 1];
  __shared__ Z gb[8][UPD_KMAX];
  __shared__ int st[UPD_KMAX];
  const int tx = threadIdx.x, ty = threadIdx.y, tid = ty * 32 + tx;
  for (int l = tid; l < m; l += 256) st[l] = sites[(long long)c * UPD_KMAX + l];
  for (int e = tid; e < m * m; e += 256)
    Ws[e / m][e % m] = A::mk(W[(((long long)c * 2 + f) * UPD_KMAX + e / m) * UPD_KMAX + e % m]);
  __syncthreads();
  const int col = blockIdx.x * 8 + ty;
  const zd* Gf = Gv + (long long)c * sG + (long long)f * N * N;
  const long long xy = ((long long)c * 2 + f) * N * UPD_KMAX;
  if (col < N && tx < m) {
    const int s = st[tx];
    const int s2 = sites2 ? sites2[(long long)c * UPD_KMAX + tx] : -1;
    if (s2 < 0) {
      X[xy + col + (long long)tx * N] = Gf[col + (long long)s * N];  // row `col` of X
      gb[ty][tx] = A::mk(zsub(zmk(s == col ? 1.0 : 0.0, 0.0), Gf[s + (long long)col * N]));
    } else {
      const double ca = coefs[2 * ((long long)c * UPD_KMAX + tx)], cb = coefs[2 * ((long long)c * UPD_KMAX + tx) + 1];
      X[xy + col + (long long)tx * N] =
          zadd(zscale(Gf[col + (long long)s * N], ca), zscale(Gf[col + (long long)s2 * N], cb));
      const double e = (s == col ? ca : 0.0) + (s2 == col ? cb : 0.0);
      gb[ty][tx] = A::mk(zsub(zmk(e, 0.0), zadd(zscale(Gf[s + (long long)col * N], ca),
                                                zscale(Gf[s2 + (long long)col * N], cb))));
    }
  }
  __syncthreads();
  if (col < N && tx < m) {
    Z y = A::zero();
    for (int l2 = 0; l2 < m; ++l2) y = A::mac(y, Ws[tx][l2], gb[ty][l2]);
    Y[xy + tx + (long long)col * UPD_KMAX] = A::wide(y);
  }
}

