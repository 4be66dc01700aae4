// CPU oracle for the finite-temperature AFQMC sweep -- TEST INFRASTRUCTURE.
//
// This file restates ALF's default (no STAB flag) sequential sweep on the CPU,
// calling the same LAPACK/BLAS routines the Fortran calls (ZGEQP3, ZUNGQR,
// ZUNMQR, ZTRSM, ZTRMM, ZGETRF, ZLAPMR/ZLAPMT, ZLARCM/ZLACRM, ZGEMM), which are
// resolved at run time from an OpenBLAS shared library (dlopen).  The GPU
// library's results are compared with it, and it is the timed CPU baseline; the
// product never links, loads or calls it.
//
// Reference files followed (paths inside the ALF tree):
//   Prog/main.F90:446-457, 589-631, 714-887       init chain and sweep block
//   Prog/Wrapgr_mod.F90:81-243                    WRAPGRUP / WRAPGRDO
//   Prog/upgrade_mod.F90:105-302                  Upgrade2
//   Prog/Operator_mod.F90:160-181, 555-951        Op_phase, Op_mmultL/R, Op_Wrapup/do
//   Prog/Hop_mod.F90:143-250, OpTTypes_mod.F90:150-201   exp(-dtau T) products
//   Libraries/Modules/Mat_subroutines_mod.F90:1225-1418 dense ZDSLSYMM (ZLARCM/ZLACRM)
//   Prog/udv_state_mod.F90:320-345, 448-582       reset / decompose
//   Prog/QDRP_decompose_mod.F90:60-126            pivoted QR + D, pivot phase
//   Prog/wrapur_mod.F90:101-124, wrapul_mod.F90:108-131
//   Prog/cgr1_mod.F90:174-447                     CGR (default branch)
//   Prog/tau_m_mod.F90:56-263, cgr2_2_mod.F90:55-73, 155-191, 317-425
//   Prog/control_mod.F90:207-320                  precision statistics
//   Prog/Fields_mod.F90:112-217                   phi / gamma / flip
//   Libraries/Modules/random_wrap_mod.F90:159-168 nranf
//   Libraries/Modules/mymats_mod.F90:683-704, 1334-1366  COMPARE_C, DET_C
//   Prog/Hamiltonians/Hamiltonian_Hubbard_smod.F90:695-801  Obs_scal of ham%Obser (Kin, Pot, Part, Ener)
//
// Storage: column-major complex128 (Fortran layout).  Indices are 0-based.
#include <complex>
#include <vector>
#include <cstring>
#include <cstdint>
#include <cmath>
#include <string>
#include <dlfcn.h>

using zc = std::complex<double>;
using std::vector;

// ---------------------------------------------------------------------------
// LAPACK / BLAS resolved at run time (Fortran ABI; hidden string lengths last)
// ---------------------------------------------------------------------------
typedef void (*zgemm_f)(const char*, const char*, const int*, const int*, const int*, const zc*,
                        const zc*, const int*, const zc*, const int*, const zc*, zc*, const int*, size_t, size_t);
typedef void (*zgeqp3_f)(const int*, const int*, zc*, const int*, int*, zc*, zc*, const int*, double*, int*);
typedef void (*zungqr_f)(const int*, const int*, const int*, zc*, const int*, const zc*, zc*, const int*, int*);
typedef void (*zunmqr_f)(const char*, const char*, const int*, const int*, const int*, const zc*, const int*,
                         const zc*, zc*, const int*, zc*, const int*, int*, size_t, size_t);
typedef void (*ztrxm_f)(const char*, const char*, const char*, const char*, const int*, const int*, const zc*,
                        const zc*, const int*, zc*, const int*, size_t, size_t, size_t, size_t);
typedef void (*zgetrf_f)(const int*, const int*, zc*, const int*, int*, int*);
typedef void (*zlapm_f)(const int*, const int*, const int*, zc*, const int*, int*);
typedef void (*zlarcm_f)(const int*, const int*, const double*, const int*, const zc*, const int*, zc*,
                         const int*, double*);
typedef void (*zlacrm_f)(const int*, const int*, const zc*, const int*, const double*, const int*, zc*,
                         const int*, double*);
typedef void (*setthreads_f)(int);

static struct {
  void* h = nullptr;
  zgemm_f zgemm; zgeqp3_f zgeqp3; zungqr_f zungqr; zunmqr_f zunmqr; ztrxm_f ztrsm, ztrmm;
  zgetrf_f zgetrf; zlapm_f zlapmr, zlapmt; zlarcm_f zlarcm; zlacrm_f zlacrm; setthreads_f setthreads;
} LA;

extern "C" int oracle_load_lapack(const char* path, const char* prefix) {
  if (LA.h) return 0;
  void* h = dlopen(path, RTLD_NOW | RTLD_LOCAL);
  if (!h) return 1;
  std::string p(prefix ? prefix : "");
  auto sym = [&](const char* n) { return dlsym(h, (p + n).c_str()); };
  LA.zgemm = (zgemm_f)sym("zgemm_");
  LA.zgeqp3 = (zgeqp3_f)sym("zgeqp3_");
  LA.zungqr = (zungqr_f)sym("zungqr_");
  LA.zunmqr = (zunmqr_f)sym("zunmqr_");
  LA.ztrsm = (ztrxm_f)sym("ztrsm_");
  LA.ztrmm = (ztrxm_f)sym("ztrmm_");
  LA.zgetrf = (zgetrf_f)sym("zgetrf_");
  LA.zlapmr = (zlapm_f)sym("zlapmr_");
  LA.zlapmt = (zlapm_f)sym("zlapmt_");
  LA.zlarcm = (zlarcm_f)sym("zlarcm_");
  LA.zlacrm = (zlacrm_f)sym("zlacrm_");
  LA.setthreads = (setthreads_f)sym("openblas_set_num_threads");
  if (!LA.zgemm || !LA.zgeqp3 || !LA.zungqr || !LA.zunmqr || !LA.ztrsm || !LA.ztrmm || !LA.zgetrf ||
      !LA.zlapmr || !LA.zlapmt || !LA.zlarcm || !LA.zlacrm)
    return 2;
  LA.h = h;
  return 0;
}

extern "C" void oracle_set_threads(int n) {
  if (LA.setthreads) LA.setthreads(n);
}

static void gemm(char ta, char tb, int m, int n, int k, zc alpha, const zc* A, int lda, const zc* B, int ldb,
                 zc beta, zc* C, int ldc) {
  LA.zgemm(&ta, &tb, &m, &n, &k, &alpha, A, &lda, B, &ldb, &beta, C, &ldc, 1, 1);
}

// ---------------------------------------------------------------------------
// Field tables (Prog/Fields_mod.F90:270-301)
// ---------------------------------------------------------------------------
static const double SQ6 = 2.449489742783178098197284074705891391965947480656670128432692567;
static double phi_st(int s, int type) {
  if (type == 1) return (double)s;
  const double a = std::sqrt(2.0 * (3.0 + SQ6)), b = std::sqrt(2.0 * (3.0 - SQ6));
  switch (s) { case -2: return -a; case -1: return -b; case 1: return b; case 2: return a; }
  return 0.0;
}
static double gama_st(int s, int type) {
  if (type == 1) return 1.0;
  return (s == 2 || s == -2) ? 1.0 - SQ6 / 3.0 : 1.0 + SQ6 / 3.0;
}
static int flip_st(int s, int k /*1..3*/) {
  static const int tab[5][3] = {{-1, 1, 2}, {1, 2, -2}, {0, 0, 0}, {2, -2, -1}, {-2, -1, 1}};
  return tab[s + 2][k - 1];
}
// nranf (Libraries/Modules/random_wrap_mod.F90:159-168): nint(r*N + 0.5), clamped.
static int nranf(double r, int N) {
  double y = r * (double)N;
  y = y + 0.5;
  long v = std::lround(y);
  if (v < 1) v = 1;
  if (v > N) v = N;
  return (int)v;
}

// ---------------------------------------------------------------------------
// State
// ---------------------------------------------------------------------------
struct UDV {
  vector<zc> U, V, D;
  char side;
  void alloc(int N) { U.assign((size_t)N * N, 0.0); V.assign((size_t)N * N, 0.0); D.assign(N, 1.0); }
  void reset(int N, char s) {  // udv_state_mod.F90:320-345
    side = s;
    std::fill(U.begin(), U.end(), zc(0.0));
    std::fill(V.begin(), V.end(), zc(0.0));
    for (int i = 0; i < N; ++i) { U[i + (size_t)i * N] = 1.0; V[i + (size_t)i * N] = 1.0; D[i] = 1.0; }
  }
};

struct Stats {
  int64_t n_prop, n_acc, n_prop_eff, n_acc_eff;
  int64_t ncg; double xmeanG_sum, xmaxG, xmaxP;
  int64_t ncg_tau; double xmean_tau_sum, xmax_tau;
};

struct SweepCursor {
  bool active = false;
  int phase = 0, ntau = 0, NST = 1;
};

struct Oracle {
  int N, F, NSUN, M, L, Nwrap, Nstm, ltau;
  SweepCursor cur;
  vector<int> stab_nt;
  vector<double> expT, expTinv;  // F x N x N
  // checkerboard Op_T (Predefined_Hop_mod.F90:1773-1839): Ncheck two-site bond operators per
  // flavour in Op_T order, P [F][Ncheck][2], mat = exp(g O) and inv = exp(-g O) [F][Ncheck][4]
  int ncheck = 0;
  vector<int> cb_P;
  vector<double> cb_mat, cb_inv;
  // vertices, k = nf*M + n
  vector<int> op_n, op_nz, op_diag, op_type, op_P;
  vector<zc> op_g, op_alpha, op_U, op_Eexp, op_Mexp;
  vector<double> op_E;
  vector<int8_t> f;  // f[nt*M + n], nt = 0..L-1 is Fortran nt = 1..L
  vector<zc> G;      // F x N x N
  vector<UDV> udvl, udvr, udvst;  // udvst[(nst-1)*F + nf], nst = 1..Nstm
  zc phase;
  Stats st;
  // scratch
  vector<zc> tmp, tmp2;
  vector<double> rwork;
  // recording (optional, caller-owned)
  int8_t* rec_acc = nullptr;
  zc* rec_ratio = nullptr;
  zc* rec_G = nullptr;       // per stabilisation point: F*N*N (fresh G after CGR)
  zc* rec_Gwrap = nullptr;   // per stabilisation point: F*N*N (wrapped G before CGR)
  zc* rec_phase = nullptr;   // per stabilisation point
  int rec_visit = 0, rec_stab = 0;
  // time displaced (TAU_M)
  void (*tau_cb)(void*, int, const zc*, const zc*, const zc*, const zc*, zc) = nullptr;
  void* tau_ctx = nullptr;
  // equal-time measurements (ham%Obser, main.F90:757-772 and 788-803): G of all flavours
  void (*eq_cb)(void*, int, const zc*, zc) = nullptr;
  void* eq_ctx = nullptr;
  // scalar observables of ham%Obser (Hubbard): H F x N x N column-major, U per site
  vector<double> obsH, obsU;
  zc obs_sum[4] = {0.0, 0.0, 0.0, 0.0};  // Kin, Pot, Part, Ener, each times ZP ZS
  double obs_sign = 0.0;
  int64_t obs_count = 0;

  zc* Gf(int nf) { return G.data() + (size_t)nf * N * N; }
  int fval(int n, int nt1 /*1-based*/) const { return f[(size_t)(nt1 - 1) * M + n]; }
};

// Obs_scal part of the Hubbard ham%Obser (Prog/Hamiltonians/Hamiltonian_Hubbard_smod.F90:695-801,
// kinetic term as Predefined_Hoppings_Compute_Kin for a dense hopping matrix):
// GRC(i,j) = delta_ij - G(j,i); ZP = Phase / Re(Phase); ZS = sign(Re(Phase));
// Kin = N_SUN sum_f sum_ij H_f(i,j) GRC_f(i,j); Pot = sum_i U_i GRC_1(i,i) GRC_dec(i,i);
// Part = N_SUN sum_f sum_i GRC_f(i,i); Ener = Kin + Pot.
static void obs_scal(Oracle& o) {
  if (o.obsH.empty()) return;
  const int N = o.N;
  const size_t NN = (size_t)N * N;
  const double re = o.phase.real();
  const zc zp = o.phase / re;
  const double zs = re > 0 ? 1.0 : (re < 0 ? -1.0 : 0.0);
  zc kin = 0.0, pot = 0.0, part = 0.0;
  for (int nf = 0; nf < o.F; ++nf) {
    const zc* G = o.Gf(nf);
    const double* H = o.obsH.data() + nf * NN;
    for (int j = 0; j < N; ++j)
      for (int i = 0; i < N; ++i) {
        const zc grc = (i == j ? 1.0 : 0.0) - G[j + (size_t)i * N];
        kin += H[i + (size_t)j * N] * grc;
      }
    for (int i = 0; i < N; ++i) part += 1.0 - G[i + (size_t)i * N];
  }
  const int dec = o.F == 2 ? 1 : 0;
  for (int i = 0; i < N; ++i)
    pot += o.obsU[i] * (1.0 - o.Gf(0)[i + (size_t)i * N]) * (1.0 - o.Gf(dec)[i + (size_t)i * N]);
  kin *= (double)o.NSUN;
  part *= (double)o.NSUN;
  const zc w = zp * zs;
  o.obs_sum[0] += kin * w; o.obs_sum[1] += pot * w; o.obs_sum[2] += part * w; o.obs_sum[3] += (kin + pot) * w;
  o.obs_sign += zs;
  o.obs_count++;
}

// ---------------------------------------------------------------------------
// Hop_mod (dense real Op_T; ZDSLSYMM dense branch uses ZLARCM / ZLACRM)
// ---------------------------------------------------------------------------
// Summation-order variant: 0 = OpenBLAS ZLARCM/ZLACRM (as the reference links), 1 = plain loops.
// Used only to measure how much two valid BLAS builds of the reference differ.
static int g_variant = 0;
extern "C" void oracle_set_variant(int v) { g_variant = v; }

static void lmult_real(Oracle& o, const double* A, zc* X) {  // X = A * X
  int N = o.N;
  o.tmp.assign(X, X + (size_t)N * N);
  if (g_variant == 1) {
    for (int j = 0; j < N; ++j)
      for (int i = 0; i < N; ++i) {
        double re = 0.0, im = 0.0;
        for (int k = N - 1; k >= 0; --k) { re += A[i + (size_t)k * N] * o.tmp[k + (size_t)j * N].real(); im += A[i + (size_t)k * N] * o.tmp[k + (size_t)j * N].imag(); }
        X[i + (size_t)j * N] = zc(re, im);
      }
    return;
  }
  o.rwork.resize((size_t)2 * N * N);
  LA.zlarcm(&N, &N, A, &N, o.tmp.data(), &N, X, &N, o.rwork.data());
}
static void rmult_real(Oracle& o, const double* A, zc* X) {  // X = X * A
  int N = o.N;
  o.tmp.assign(X, X + (size_t)N * N);
  if (g_variant == 1) {
    for (int j = 0; j < N; ++j)
      for (int i = 0; i < N; ++i) {
        double re = 0.0, im = 0.0;
        for (int k = N - 1; k >= 0; --k) { re += o.tmp[i + (size_t)k * N].real() * A[k + (size_t)j * N]; im += o.tmp[i + (size_t)k * N].imag() * A[k + (size_t)j * N]; }
        X[i + (size_t)j * N] = zc(re, im);
      }
    return;
  }
  o.rwork.resize((size_t)2 * N * N);
  LA.zlacrm(&N, &N, o.tmp.data(), &N, A, &N, X, &N, o.rwork.data());
}
static const double* mat(Oracle& o, int nf) { return o.expT.data() + (size_t)nf * o.N * o.N; }
static const double* inv(Oracle& o, int nf) { return o.expTinv.data() + (size_t)nf * o.N * o.N; }
// One checkerboard bond operator (2 x 2, column-major E) on rows (X <- E X) or columns (X <- X E)
// P1, P2 of X: the two-site RealExpOpT lmult / rmult (OpTTypes_mod.F90:135-304).
static void bond_l(Oracle& o, zc* X, int nf, int nc, const vector<double>& E) {
  const int N = o.N, a = o.cb_P[2 * ((size_t)nf * o.ncheck + nc)], b = o.cb_P[2 * ((size_t)nf * o.ncheck + nc) + 1];
  const double* e = E.data() + 4 * ((size_t)nf * o.ncheck + nc);
  for (int j = 0; j < N; ++j) {
    const zc xa = X[a + (size_t)j * N], xb = X[b + (size_t)j * N];
    X[a + (size_t)j * N] = e[0] * xa + e[2] * xb;
    X[b + (size_t)j * N] = e[1] * xa + e[3] * xb;
  }
}
static void bond_r(Oracle& o, zc* X, int nf, int nc, const vector<double>& E) {
  const int N = o.N, a = o.cb_P[2 * ((size_t)nf * o.ncheck + nc)], b = o.cb_P[2 * ((size_t)nf * o.ncheck + nc) + 1];
  const double* e = E.data() + 4 * ((size_t)nf * o.ncheck + nc);
  for (int i = 0; i < N; ++i) {
    const zc xa = X[i + (size_t)a * N], xb = X[i + (size_t)b * N];
    X[i + (size_t)a * N] = xa * e[0] + xb * e[1];
    X[i + (size_t)b * N] = xa * e[2] + xb * e[3];
  }
}
// Hop_mod.F90:143-250 (dense: one Op_T; checkerboard: the bond operators in the order of each routine)
static void hop_mmthr(Oracle& o, zc* X, int nf) {  // B_T X: nc = Ncheck .. 1, lmult
  if (!o.ncheck) return lmult_real(o, mat(o, nf), X);
  for (int nc = o.ncheck - 1; nc >= 0; --nc) bond_l(o, X, nf, nc, o.cb_mat);
}
static void hop_mmthr_m1(Oracle& o, zc* X, int nf) {  // B_T^-1 X: nc = 1 .. Ncheck, lmultinv
  if (!o.ncheck) return lmult_real(o, inv(o, nf), X);
  for (int nc = 0; nc < o.ncheck; ++nc) bond_l(o, X, nf, nc, o.cb_inv);
}
static void hop_mmthl(Oracle& o, zc* X, int nf) {  // X B_T: nc = 1 .. Ncheck, rmult
  if (!o.ncheck) return rmult_real(o, mat(o, nf), X);
  for (int nc = 0; nc < o.ncheck; ++nc) bond_r(o, X, nf, nc, o.cb_mat);
}
static void hop_mmthl_m1(Oracle& o, zc* X, int nf) {  // X B_T^-1: nc = Ncheck .. 1, rmultinv
  if (!o.ncheck) return rmult_real(o, inv(o, nf), X);
  for (int nc = o.ncheck - 1; nc >= 0; --nc) bond_r(o, X, nf, nc, o.cb_inv);
}
static void hop_mmthlc(Oracle& o, zc* X, int nf) {  // nc = 1 .. Ncheck, lmult (B_T^T X for symmetric bonds)
  if (!o.ncheck) return lmult_real(o, mat(o, nf), X);
  for (int nc = 0; nc < o.ncheck; ++nc) bond_l(o, X, nf, nc, o.cb_mat);
}

// ---------------------------------------------------------------------------
// Operator_mod small x large products (ZSLGEMM semantics, N_op <= 2)
// ---------------------------------------------------------------------------
static inline zc opA(const zc* A, int n, int i, int j, char cop) {  // op(A)(i,j), A col-major n x n
  if (cop == 'n' || cop == 'N') return A[i + j * n];
  if (cop == 't' || cop == 'T') return A[j + i * n];
  return std::conj(A[j + i * n]);
}
// Mat(P,:) = op(A) * Mat(P,:)
static void sl_left(int N, int n, const int* P, const zc* A, char cop, zc* Mat) {
  for (int c = 0; c < N; ++c) {
    zc z[2];
    for (int a = 0; a < n; ++a) z[a] = Mat[P[a] + (size_t)c * N];
    for (int a = 0; a < n; ++a) {
      zc s = 0.0;
      for (int b = 0; b < n; ++b) s += opA(A, n, a, b, cop) * z[b];
      Mat[P[a] + (size_t)c * N] = s;
    }
  }
}
// Mat(:,P) = Mat(:,P) * op(A)
static void sl_right(int N, int n, const int* P, const zc* A, char cop, zc* Mat) {
  for (int r = 0; r < N; ++r) {
    zc z[2];
    for (int a = 0; a < n; ++a) z[a] = Mat[r + (size_t)P[a] * N];
    for (int b = 0; b < n; ++b) {
      zc s = 0.0;
      for (int a = 0; a < n; ++a) s += z[a] * opA(A, n, a, b, cop);
      Mat[r + (size_t)P[b] * N] = s;
    }
  }
}
static inline zc eexp(const Oracle& o, int k, int m, int s) { return o.op_Eexp[((size_t)k * 2 + m) * 5 + (s + 2)]; }
static inline const zc* opU(const Oracle& o, int k) { return o.op_U.data() + (size_t)k * 4; }
static inline const zc* mexp(const Oracle& o, int k, int s) { return o.op_Mexp.data() + ((size_t)k * 5 + (s + 2)) * 4; }
static inline const int* opP(const Oracle& o, int k) { return o.op_P.data() + (size_t)k * 2; }

static void scale_row(int N, zc* Mat, int r, zc a) { for (int c = 0; c < N; ++c) Mat[r + (size_t)c * N] *= a; }
static void scale_col(int N, zc* Mat, int c, zc a) { for (int r = 0; r < N; ++r) Mat[r + (size_t)c * N] *= a; }

// Op_Wrapup (Prog/Operator_mod.F90:743-835), types 1,2 without g(t).
static void op_wrapup(Oracle& o, zc* Mat, int k, int s, int ntype) {
  int N = o.N, n = o.op_n[k];
  const int* P = opP(o, k);
  if (ntype == 1) {
    if (o.op_diag[k]) {
      for (int I = 0; I < n; ++I) scale_row(N, Mat, P[I], eexp(o, k, I, s));
      for (int I = 0; I < n; ++I) scale_col(N, Mat, P[I], eexp(o, k, I, -s));
    } else {
      zc VH1[4];
      const zc* U = opU(o, k);
      for (int i = 0; i < n; ++i) for (int r = 0; r < n; ++r) VH1[r + i * n] = U[r + i * n] * eexp(o, k, i, -s);
      sl_right(N, n, P, VH1, 'n', Mat);
      for (int i = 0; i < n; ++i) for (int r = 0; r < n; ++r) VH1[r + i * n] = eexp(o, k, i, s) * std::conj(U[r + i * n]);
      sl_left(N, n, P, VH1, 'T', Mat);
    }
  } else if (ntype == 2 && !o.op_diag[k]) {
    sl_left(N, n, P, opU(o, k), 'n', Mat);
    sl_right(N, n, P, opU(o, k), 'c', Mat);
  }
}
// Op_Wrapdo (Prog/Operator_mod.F90:862-951)
static void op_wrapdo(Oracle& o, zc* Mat, int k, int s, int ntype) {
  int N = o.N, n = o.op_n[k];
  const int* P = opP(o, k);
  if (ntype == 1) {
    if (o.op_diag[k]) {
      for (int I = 0; I < n; ++I) scale_row(N, Mat, P[I], eexp(o, k, I, -s));
      for (int I = 0; I < n; ++I) scale_col(N, Mat, P[I], eexp(o, k, I, s));
    } else {
      zc VH1[4];
      const zc* U = opU(o, k);
      for (int i = 0; i < n; ++i) for (int r = 0; r < n; ++r) VH1[r + i * n] = U[r + i * n] * eexp(o, k, i, -s);
      sl_left(N, n, P, VH1, 'n', Mat);
      for (int i = 0; i < n; ++i) for (int r = 0; r < n; ++r) VH1[r + i * n] = eexp(o, k, i, s) * std::conj(U[r + i * n]);
      sl_right(N, n, P, VH1, 'T', Mat);
    }
  } else if (ntype == 2 && !o.op_diag[k]) {
    sl_right(N, n, P, opU(o, k), 'n', Mat);
    sl_left(N, n, P, opU(o, k), 'c', Mat);
  }
}
// Op_mmultR (Prog/Operator_mod.F90:648-717): Mat = op(exp(g phi O)) * Mat
static void op_mmultR(Oracle& o, zc* Mat, int k, int s, char cop) {
  if (std::abs(o.op_g[k]) < 1e-12) return;
  int N = o.N, n = o.op_n[k];
  const int* P = opP(o, k);
  if (o.op_diag[k]) {
    for (int I = 0; I < n; ++I) {
      zc a = eexp(o, k, I, s);
      if (cop == 'c' || cop == 'C') a = std::conj(a);
      scale_row(N, Mat, P[I], a);
    }
  } else {
    sl_left(N, n, P, mexp(o, k, s), cop, Mat);
  }
}
// Op_mmultL (Prog/Operator_mod.F90:555-623): Mat = Mat * op(exp(sign g phi O))
static void op_mmultL(Oracle& o, zc* Mat, int k, int s0, char cop, int sign) {
  if (std::abs(o.op_g[k]) < 1e-12) return;
  int N = o.N, n = o.op_n[k], s = sign * s0;
  const int* P = opP(o, k);
  if (o.op_diag[k]) {
    for (int I = 0; I < n; ++I) {
      zc a = eexp(o, k, I, s);
      if (cop == 'c' || cop == 'C') a = std::conj(a);
      scale_col(N, Mat, P[I], a);
    }
  } else {
    sl_right(N, n, P, mexp(o, k, s), cop, Mat);
  }
}
// Op_phase (Prog/Operator_mod.F90:160-181)
static void op_phase(Oracle& o, zc& ph, int nf) {
  for (int n = 0; n < o.M; ++n) {
    int k = nf * o.M + n;
    for (int nt = 1; nt <= o.L; ++nt) {
      double angle = std::imag(o.op_g[k] * o.op_alpha[k] * phi_st(o.fval(n, nt), o.op_type[k]));
      ph = ph * zc(std::cos(angle), std::sin(angle));
    }
  }
}

// ---------------------------------------------------------------------------
// Upgrade2 (Prog/upgrade_mod.F90:105-302), mode "Final", S0 = T0 ratio = 1
// ---------------------------------------------------------------------------
static bool upgrade2(Oracle& o, int n, int nt1, int hs_new, double r_metro, zc* ratio_out) {
  int F = o.F, N = o.N;
  int hs_old = o.fval(n, nt1);
  zc Ratio[2];
  zc Delta[2][2];
  for (int nf = 0; nf < F; ++nf) {
    int k = nf * o.M + n;
    const int* P = opP(o, k);
    zc Z1 = o.op_g[k] * (phi_st(hs_new, o.op_type[k]) - phi_st(hs_old, o.op_type[k]));
    int d = o.op_nz[k];
    zc Mat[2][2];
    zc* G = o.Gf(nf);
    for (int m = 0; m < d; ++m) {
      zc myexp = std::exp(Z1 * o.op_E[(size_t)k * 2 + m]);
      zc Z = myexp - 1.0;
      Delta[nf][m] = Z;
      for (int a = 0; a < d; ++a) Mat[a][m] = -Z * G[P[a] + (size_t)P[m] * N];
      Mat[m][m] = myexp + Mat[m][m];
    }
    zc D;
    if (d == 0) D = 1.0;
    else if (d == 1) D = Mat[0][0];
    else {
      zc s1 = Mat[0][0] * Mat[1][1], s2 = Mat[1][0] * Mat[0][1];
      if (std::abs(s1) > std::abs(s2)) D = s1 * (1.0 - s2 / s1);
      else D = s2 * (s1 / s2 - 1.0);
    }
    Ratio[nf] = D * std::exp(Z1 * o.op_alpha[k]);
  }
  zc Ratiotot = 1.0;
  for (int nf = 0; nf < F; ++nf) Ratiotot *= Ratio[nf];
  int type = o.op_type[n];
  Ratiotot = std::pow(Ratiotot, (double)o.NSUN) * gama_st(hs_new, type) / gama_st(hs_old, type);
  if (ratio_out) *ratio_out = Ratiotot;
  double Weight = std::abs(std::real(o.phase * Ratiotot) / std::real(o.phase));
  bool toggle = Weight > r_metro;
  if (toggle) {
    o.phase = o.phase * Ratiotot / std::sqrt(Ratiotot * std::conj(Ratiotot));
    for (int nf = 0; nf < F; ++nf) {
      int k = nf * o.M + n;
      const int* P = opP(o, k);
      int d = o.op_nz[k];
      if (d == 0) continue;
      zc* G = o.Gf(nf);
      vector<zc> u((size_t)N * d, 0.0), v((size_t)N * d, 0.0), xv((size_t)N * d, 0.0), yv((size_t)N * d, 0.0);
      for (int a = 0; a < d; ++a) {
        u[P[a] + (size_t)a * N] = Delta[nf][a];
        for (int i = 0; i < N; ++i) v[i + (size_t)a * N] = -G[P[a] + (size_t)i * N];
        v[P[a] + (size_t)a * N] = 1.0 - G[P[a] + (size_t)P[a] * N];
      }
      int i0 = P[0];
      xv[i0] = u[i0] / (1.0 + v[i0] * u[i0]);
      for (int i = 0; i < N; ++i) yv[i] = v[i];
      for (int a = 1; a < d; ++a) {
        for (int i = 0; i < N; ++i) { xv[i + (size_t)a * N] = u[i + (size_t)a * N]; yv[i + (size_t)a * N] = v[i + (size_t)a * N]; }
        zc Z = 1.0 + u[P[a] + (size_t)a * N] * v[P[a] + (size_t)a * N];
        zc syu[2], sxv[2];
        for (int m = 0; m < a; ++m) {
          zc s1 = 0.0, s2 = 0.0;
          for (int i = 0; i < N; ++i) {
            s1 += yv[i + (size_t)m * N] * u[i + (size_t)a * N];
            s2 += xv[i + (size_t)m * N] * v[i + (size_t)a * N];
          }
          syu[m] = -s1;
          sxv[m] = -s2;
        }
        for (int i = 0; i < N; ++i) {
          zc ax = 0.0, ay = 0.0;
          for (int m = 0; m < a; ++m) { ax += xv[i + (size_t)m * N] * syu[m]; ay += yv[i + (size_t)m * N] * sxv[m]; }
          xv[i + (size_t)a * N] += ax;
          yv[i + (size_t)a * N] += ay;
        }
        for (int m = 0; m < a; ++m) Z = Z - syu[m] * sxv[m];
        Z = 1.0 / Z;
        for (int i = 0; i < N; ++i) xv[i + (size_t)a * N] *= Z;
      }
      if (o.op_n[k] == 1) {
        vector<zc> xp(G + (size_t)P[0] * N, G + (size_t)P[0] * N + N);
        zc Z = -xv[P[0]];
        for (int j = 0; j < N; ++j) {  // ZGERU
          zc t = Z * yv[j];
          zc* Gc = G + (size_t)j * N;
          for (int i = 0; i < N; ++i) Gc[i] += xp[i] * t;
        }
      } else {
        zc Zarr[4];
        for (int a = 0; a < d; ++a) for (int b = 0; b < d; ++b) Zarr[a + b * d] = xv[P[a] + (size_t)b * N];
        vector<zc> grarr((size_t)N * d), xp((size_t)N * d);
        for (int a = 0; a < d; ++a) for (int i = 0; i < N; ++i) grarr[i + (size_t)a * N] = G[i + (size_t)P[a] * N];
        gemm('N', 'N', N, d, d, 1.0, grarr.data(), N, Zarr, d, 0.0, xp.data(), N);
        gemm('N', 'T', N, N, d, -1.0, xp.data(), N, yv.data(), N, 1.0, G, N);
      }
    }
    o.f[(size_t)(nt1 - 1) * o.M + n] = (int8_t)hs_new;
  }
  o.st.n_prop++; o.st.n_prop_eff++;
  if (toggle) { o.st.n_acc++; o.st.n_acc_eff++; }
  return toggle;
}

static int visit_flip(Oracle& o, int n, int nt1, const double* u3) {
  int type = o.op_type[n];
  int old = o.fval(n, nt1);
  if (type == 1) return -old;
  return flip_st(old, nranf(u3[0], 3));
}

// WRAPGRUP (Prog/Wrapgr_mod.F90:81-156): NTAU -> NTAU+1, update slice NTAU+1
static void wrapgrup(Oracle& o, int ntau, const double* u) {
  int nt1 = ntau + 1;
  for (int nf = 0; nf < o.F; ++nf) { hop_mmthr(o, o.Gf(nf), nf); hop_mmthl_m1(o, o.Gf(nf), nf); }
  for (int n = 0; n < o.M; ++n) {
    int hs = o.fval(n, nt1);
    for (int nf = 0; nf < o.F; ++nf) op_wrapup(o, o.Gf(nf), nf * o.M + n, hs, 1);
    const double* u3 = u + (size_t)3 * n;
    int hs_new = visit_flip(o, n, nt1, u3);
    zc ratio = 0.0;
    bool acc = false;
    if (1.5 > u3[1]) acc = upgrade2(o, n, nt1, hs_new, u3[2], &ratio);
    else { o.st.n_prop_eff++; }
    if (o.rec_acc) o.rec_acc[o.rec_visit] = acc;
    if (o.rec_ratio) o.rec_ratio[o.rec_visit] = ratio;
    o.rec_visit++;
    for (int nf = 0; nf < o.F; ++nf) op_wrapup(o, o.Gf(nf), nf * o.M + n, hs, 2);
  }
}
// WRAPGRDO (Prog/Wrapgr_mod.F90:160-243): update slice NTAU, NTAU -> NTAU-1
static void wrapgrdo(Oracle& o, int ntau, const double* u) {
  for (int n = o.M - 1; n >= 0; --n) {
    int hs = o.fval(n, ntau);
    for (int nf = 0; nf < o.F; ++nf) op_wrapdo(o, o.Gf(nf), nf * o.M + n, hs, 2);
    const double* u3 = u + (size_t)3 * (o.M - 1 - n);
    int hs_new = visit_flip(o, n, ntau, u3);
    zc ratio = 0.0;
    bool acc = false;
    if (1.5 > u3[1]) acc = upgrade2(o, n, ntau, hs_new, u3[2], &ratio);
    else { o.st.n_prop_eff++; }
    if (o.rec_acc) o.rec_acc[o.rec_visit] = acc;
    if (o.rec_ratio) o.rec_ratio[o.rec_visit] = ratio;
    o.rec_visit++;
    hs = o.fval(n, ntau);
    for (int nf = 0; nf < o.F; ++nf) op_wrapdo(o, o.Gf(nf), nf * o.M + n, hs, 1);
  }
  for (int nf = 0; nf < o.F; ++nf) { hop_mmthl(o, o.Gf(nf), nf); hop_mmthr_m1(o, o.Gf(nf), nf); }
}

// ---------------------------------------------------------------------------
// QDRP_decompose (Prog/QDRP_decompose_mod.F90:60-101) and Pivot_phase (:103-126)
// ---------------------------------------------------------------------------
static void qdrp(int N, zc* A, zc* D, int* ipvt, vector<zc>& tau) {
  tau.assign(N, 0.0);
  for (int i = 0; i < N; ++i) ipvt[i] = 0;
  vector<double> rw(2 * N);
  zc wq; int lw = -1, info = 0;
  LA.zgeqp3(&N, &N, A, &N, ipvt, tau.data(), &wq, &lw, rw.data(), &info);
  lw = (int)std::real(wq);
  vector<zc> work(std::max(lw, 1));
  LA.zgeqp3(&N, &N, A, &N, ipvt, tau.data(), work.data(), &lw, rw.data(), &info);
  for (int i = 0; i < N; ++i) {
    double X = std::abs(A[i + (size_t)i * N]);
    D[i] = X;
    for (int j = i; j < N; ++j) A[i + (size_t)j * N] /= X;
  }
}
static void pivot_phase(zc& ph, const int* ipvt, int N) {
  vector<int> vis(N, 0);
  for (int i = 0; i < N; ++i) {
    if (!vis[i]) {
      int next = i, Lc = 0;
      while (!vis[next]) { Lc++; vis[next] = 1; next = ipvt[next] - 1; }
      if (Lc % 2 == 0) ph = -ph;
    }
  }
}

// decompose_UDV_state, default branch (Prog/udv_state_mod.F90:466-578)
static void decompose(int N, UDV& s) {
  for (int i = 0; i < N; ++i) for (int r = 0; r < N; ++r) s.U[r + (size_t)i * N] *= s.D[i];
  vector<int> ipvt(N);
  vector<zc> tau;
  qdrp(N, s.U.data(), s.D.data(), ipvt.data(), tau);
  zc ph = 1.0;
  for (int i = 0; i < N; ++i) ph *= s.U[i + (size_t)i * N];
  pivot_phase(ph, ipvt.data(), N);
  bool left = (s.side == 'L' || s.side == 'l');
  if (left) ph = std::conj(ph);
  zc beta = 1.0 / ph;
  for (int j = 0; j < N; ++j) s.U[(size_t)j * N] *= beta;
  int fw = 1;
  if (!left) LA.zlapmr(&fw, &N, &N, s.V.data(), &N, ipvt.data());
  else LA.zlapmt(&fw, &N, &N, s.V.data(), &N, ipvt.data());
  zc one = 1.0;
  if (!left) LA.ztrmm("L", "U", "N", "N", &N, &N, &one, s.U.data(), &N, s.V.data(), &N, 1, 1, 1, 1);
  else LA.ztrmm("R", "U", "C", "N", &N, &N, &one, s.U.data(), &N, s.V.data(), &N, 1, 1, 1, 1);
  zc wq; int lw = -1, info = 0;
  LA.zungqr(&N, &N, &N, s.U.data(), &N, tau.data(), &wq, &lw, &info);
  lw = (int)std::real(wq);
  vector<zc> work(std::max(lw, 1));
  LA.zungqr(&N, &N, &N, s.U.data(), &N, tau.data(), work.data(), &lw, &info);
  for (int r = 0; r < N; ++r) s.U[r] *= ph;
}

// WRAPUR (Prog/wrapur_mod.F90:101-124)
static void wrapur(Oracle& o, int ntau, int ntau1, vector<UDV>& udvr) {
  for (int nf = 0; nf < o.F; ++nf) {
    for (int nt = ntau + 1; nt <= ntau1; ++nt) {
      hop_mmthr(o, udvr[nf].U.data(), nf);
      for (int n = 0; n < o.M; ++n) op_mmultR(o, udvr[nf].U.data(), nf * o.M + n, o.fval(n, nt), 'n');
    }
    decompose(o.N, udvr[nf]);
  }
}
// WRAPUL (Prog/wrapul_mod.F90:108-131)
static void wrapul(Oracle& o, int ntau1, int ntau, vector<UDV>& udvl) {
  for (int nf = 0; nf < o.F; ++nf) {
    for (int nt = ntau1; nt >= ntau + 1; --nt) {
      for (int n = o.M - 1; n >= 0; --n) op_mmultR(o, udvl[nf].U.data(), nf * o.M + n, o.fval(n, nt), 'c');
      hop_mmthlc(o, udvl[nf].U.data(), nf);
    }
    decompose(o.N, udvl[nf]);
  }
}

// DET_C (Libraries/Modules/mymats_mod.F90:1334-1366); destroys A
static zc det_c(int N, zc* A) {
  vector<int> ipiv(N, 0);
  int info = 0;
  LA.zgetrf(&N, &N, A, &N, ipiv.data(), &info);
  zc d = 1.0;
  for (int i = 0; i < N; ++i) d *= A[i + (size_t)i * N];
  int sgn = 1;
  for (int i = 0; i < N; ++i) if (ipiv[i] != i + 1) sgn = -sgn;
  return sgn == -1 ? -d : d;
}

// CGR default branch (Prog/cgr1_mod.F90:174-447)
static void cgr(int N, zc& phase, int nvar, zc* GR, const UDV& ur, const UDV& ul) {
  size_t NN = (size_t)N * N;
  vector<zc> TPUP(NN), RHS(NN), DUP(N), tau;
  vector<int> ipvt(N);
  gemm('C', 'N', N, N, N, 1.0, ur.U.data(), N, ul.U.data(), N, 0.0, RHS.data(), N);
  gemm('N', 'N', N, N, N, 1.0, ur.V.data(), N, ul.V.data(), N, 0.0, TPUP.data(), N);
  for (int J = 0; J < N; ++J)
    for (int I = 0; I < N; ++I) TPUP[I + (size_t)J * N] = ur.D[I] * TPUP[I + (size_t)J * N] * ul.D[J];
  for (size_t i = 0; i < NN; ++i) TPUP[i] += RHS[i];
  phase = std::conj(det_c(N, RHS.data()));
  phase = phase / std::abs(phase);
  if (nvar != 1) {
    vector<zc> t(NN);
    for (int J = 0; J < N; ++J) for (int I = 0; I < N; ++I) t[J + (size_t)I * N] = std::conj(TPUP[I + (size_t)J * N]);
    TPUP.swap(t);
  }
  qdrp(N, TPUP.data(), DUP.data(), ipvt.data(), tau);
  pivot_phase(phase, ipvt.data(), N);
  for (int i = 0; i < N; ++i) {
    zc Z = tau[i];
    zc r = TPUP[i + (size_t)i * N];
    if (nvar == 1) phase = phase * r / std::abs(r);
    else { phase = phase * std::conj(r) / std::abs(r); Z = std::conj(Z); }
    if (Z != zc(0.0)) {
      double X = std::abs(Z);
      Z = 1.0 - 2.0 * (Z / X) * (std::real(Z) / X);
      phase = phase * Z / std::abs(Z);
    }
  }
  int info = 0, lw = -1;
  zc wq;
  zc one = 1.0;
  int bw = 0;
  if (nvar == 1) {
    for (int J = 0; J < N; ++J) for (int I = 0; I < N; ++I) RHS[I + (size_t)J * N] = std::conj(ur.U[J + (size_t)I * N]);
    LA.zunmqr("L", "C", &N, &N, &N, TPUP.data(), &N, tau.data(), RHS.data(), &N, &wq, &lw, &info, 1, 1);
    lw = (int)std::real(wq);
    vector<zc> work(std::max(lw, 1));
    LA.zunmqr("L", "C", &N, &N, &N, TPUP.data(), &N, tau.data(), RHS.data(), &N, work.data(), &lw, &info, 1, 1);
    for (int J = 0; J < N; ++J) for (int I = 0; I < N; ++I) RHS[I + (size_t)J * N] = RHS[I + (size_t)J * N] / DUP[I];
    LA.ztrsm("L", "U", "N", "N", &N, &N, &one, TPUP.data(), &N, RHS.data(), &N, 1, 1, 1, 1);
    LA.zlapmr(&bw, &N, &N, RHS.data(), &N, ipvt.data());
    gemm('N', 'N', N, N, N, 1.0, ul.U.data(), N, RHS.data(), N, 0.0, GR, N);
  } else {
    RHS.assign(ul.U.begin(), ul.U.end());
    LA.zunmqr("R", "N", &N, &N, &N, TPUP.data(), &N, tau.data(), RHS.data(), &N, &wq, &lw, &info, 1, 1);
    lw = (int)std::real(wq);
    vector<zc> work(std::max(lw, 1));
    LA.zunmqr("R", "N", &N, &N, &N, TPUP.data(), &N, tau.data(), RHS.data(), &N, work.data(), &lw, &info, 1, 1);
    for (int J = 0; J < N; ++J) {
      double sv = 1.0 / std::real(DUP[J]);
      for (int I = 0; I < N; ++I) RHS[I + (size_t)J * N] = RHS[I + (size_t)J * N] * sv;
    }
    LA.ztrsm("R", "U", "C", "N", &N, &N, &one, TPUP.data(), &N, RHS.data(), &N, 1, 1, 1, 1);
    LA.zlapmt(&bw, &N, &N, RHS.data(), &N, ipvt.data());
    gemm('N', 'C', N, N, N, 1.0, RHS.data(), N, ur.U.data(), N, 0.0, GR, N);
  }
}

// COMPARE_C (mymats_mod.F90:683-704)
static void compare(int N, const zc* A, const zc* B, double& xmax, double& xmean) {
  xmax = 0.0; xmean = 0.0;
  for (int I = 0; I < N; ++I)
    for (int J = 0; J < N; ++J) {
      double d = std::abs(A[I + (size_t)J * N] - B[I + (size_t)J * N]);
      if (d > xmax) xmax = d;
      xmean += d;
    }
  xmean /= (double)N * N;
}

// Control_PrecisionG (control_mod.F90:207-298); returns 3 (ERROR_UNSTABLE_MATRIX) on XMAX > 10,
// 1 (ERROR_GENERIC) on NaN
static int precision_g(Oracle& o, const zc* A, const zc* B) {
  size_t NN = (size_t)o.N * o.N;
  for (size_t i = 0; i < NN; ++i) if (A[i] != A[i] || B[i] != B[i]) return 1;
  double xmax, xmean;
  compare(o.N, A, B, xmax, xmean);
  o.st.ncg++;
  if (xmax > 10.0) return 3;
  if (xmax > o.st.xmaxG) o.st.xmaxG = xmax;
  o.st.xmeanG_sum += xmean;
  return 0;
}

static void record_stab(Oracle& o, const vector<zc>& test) {
  size_t sz = (size_t)o.F * o.N * o.N;
  if (o.rec_G) std::memcpy(o.rec_G + (size_t)o.rec_stab * sz, o.G.data(), sz * sizeof(zc));
  if (o.rec_Gwrap) std::memcpy(o.rec_Gwrap + (size_t)o.rec_stab * sz, test.data(), sz * sizeof(zc));
  if (o.rec_phase) o.rec_phase[o.rec_stab] = o.phase;
  o.rec_stab++;
}

// Stabilisation at one point: CGR per flavour, precision, phase (main.F90:734-754 and 809-828)
static int stabilise(Oracle& o, int nvar) {
  vector<zc> zarr(o.F);
  vector<zc> test(o.G);
  for (int nf = 0; nf < o.F; ++nf) {
    zc Z1;
    cgr(o.N, Z1, nvar, o.Gf(nf), o.udvr[nf], o.udvl[nf]);
    int e = precision_g(o, o.Gf(nf), test.data() + (size_t)nf * o.N * o.N);
    if (e) return e;
    op_phase(o, Z1, nf);
    zarr[nf] = Z1;
  }
  zc Z = 1.0;
  for (int nf = 0; nf < o.F; ++nf) Z *= zarr[nf];
  Z = std::pow(Z, (double)o.NSUN);
  double X = std::abs(Z - o.phase);
  if (X > o.st.xmaxP) o.st.xmaxP = X;
  o.phase = Z;
  record_stab(o, test);
  return 0;
}

// ---------------------------------------------------------------------------
// TAU_M (Prog/tau_m_mod.F90:56-263) and CGR2_2 (Prog/cgr2_2_mod.F90:317-425)
// ---------------------------------------------------------------------------
// PROPR: AIN = B(NT1) AIN  (tau_m_mod.F90:215-236)
static void propr(Oracle& o, zc* A, int nt1, int nf) {
  hop_mmthr(o, A, nf);
  for (int n = 0; n < o.M; ++n) op_mmultR(o, A, nf * o.M + n, o.fval(n, nt1), 'n');
}
// PROPRM1: AIN = AIN B(NT1)^-1  (tau_m_mod.F90:240-263)
static void proprm1(Oracle& o, zc* A, int nt1, int nf) {
  hop_mmthl_m1(o, A, nf);
  for (int n = 0; n < o.M; ++n) op_mmultL(o, A, nf * o.M + n, o.fval(n, nt1), 'n', -1);
}

// INV_C (Libraries/Modules/mymats_mod.F90:546-593): inverse by ZGETRF + ZGETRI
typedef void (*zgetri_f)(const int*, zc*, const int*, const int*, zc*, const int*, int*);
static zgetri_f ZGETRI = nullptr;

static int zinv(int N, zc* A) {
  if (!ZGETRI) return 2;
  vector<int> ipiv(N);
  int info = 0;
  LA.zgetrf(&N, &N, A, &N, ipiv.data(), &info);
  zc wq; int lw = -1;
  ZGETRI(&N, A, &N, ipiv.data(), &wq, &lw, &info);
  lw = (int)std::real(wq);
  vector<zc> work(std::max(lw, 1));
  ZGETRI(&N, A, &N, ipiv.data(), work.data(), &lw, &info);
  return info;
}

extern "C" int oracle_load_getri(const char* path, const char* prefix) {
  void* h = dlopen(path, RTLD_NOW | RTLD_LOCAL);
  if (!h) return 1;
  std::string p(prefix ? prefix : "");
  ZGETRI = (zgetri_f)dlsym(h, (p + "zgetri_").c_str());
  return ZGETRI ? 0 : 2;
}

// get_blocks (Prog/cgr2_2_mod.F90:55-73): (A B; C D) = INP
static void get_blocks(int N, const zc* INP, zc* A, zc* B, zc* C, zc* D) {
  int N2 = 2 * N;
  for (int j = 0; j < N; ++j)
    for (int i = 0; i < N; ++i) {
      A[i + (size_t)j * N] = INP[i + (size_t)j * N2];
      D[i + (size_t)j * N] = INP[(i + N) + (size_t)(j + N) * N2];
      C[i + (size_t)j * N] = INP[(i + N) + (size_t)j * N2];
      B[i + (size_t)j * N] = INP[i + (size_t)(j + N) * N2];
    }
}

// solve_extended_System, default branch (Prog/cgr2_2_mod.F90:155-191)
static void solve_extended(int N, zc* HLP, const zc* UCT, const zc* VINV, const zc* A, const zc* D,
                           const vector<zc>& tau, const int* pivt) {
  int N2 = 2 * N;
  std::fill(HLP, HLP + (size_t)N2 * N2, zc(0.0));
  for (int j = 0; j < N; ++j)
    for (int i = 0; i < N; ++i) {
      HLP[i + (size_t)j * N2] = UCT[i + (size_t)j * N];
      HLP[(i + N) + (size_t)(j + N) * N2] = VINV[i + (size_t)j * N];
    }
  int fw = 1;
  vector<int> pv(pivt, pivt + N2);
  LA.zlapmr(&fw, &N2, &N2, HLP, &N2, pv.data());
  zc one = 1.0;
  LA.ztrsm("L", "U", "C", "N", &N2, &N2, &one, A, &N2, HLP, &N2, 1, 1, 1, 1);
  for (int J = 0; J < N2; ++J)
    for (int I = 0; I < N2; ++I) HLP[I + (size_t)J * N2] = std::conj(1.0 / D[I]) * HLP[I + (size_t)J * N2];
  int info = 0, lw = -1;
  zc wq;
  LA.zunmqr("L", "N", &N2, &N2, &N2, A, &N2, tau.data(), HLP, &N2, &wq, &lw, &info, 1, 1);
  lw = (int)std::real(wq);
  vector<zc> work(std::max(lw, 1));
  LA.zunmqr("L", "N", &N2, &N2, &N2, A, &N2, tau.data(), HLP, &N2, work.data(), &lw, &info, 1, 1);
}

// CGR2_2, default branch (Prog/cgr2_2_mod.F90:317-425).  udv2 = right state (0 -> tau),
// udv1 = stored left state (beta -> tau).
static void cgr2_2(int N, zc* GRT0, zc* GR00, zc* GRTT, zc* GR0T, const UDV& udv2, const UDV& udv1) {
  int N2 = 2 * N;
  size_t NN = (size_t)N * N, NN2 = (size_t)N2 * N2;
  vector<zc> MYU2(NN), V1INV(udv1.V), HLPB1(NN2), HLPB2(NN2, 0.0), D3(N2), tau;
  vector<int> ipvt(N2);
  for (int j = 0; j < N; ++j) for (int i = 0; i < N; ++i) MYU2[i + (size_t)j * N] = std::conj(udv2.U[j + (size_t)i * N]);
  zinv(N, V1INV.data());
  const vector<zc>& D1m = udv1.D;
  const vector<zc>& D2m = udv2.D;
  bool first = std::real(udv1.D[0]) > std::real(udv2.D[0]);
  const vector<zc>& TL = first ? V1INV : MYU2;
  const vector<zc>& BR = first ? MYU2 : V1INV;
  for (int j = 0; j < N; ++j)
    for (int i = 0; i < N; ++i) {
      HLPB2[i + (size_t)j * N2] = TL[i + (size_t)j * N];
      HLPB2[(i + N) + (size_t)(j + N) * N2] = BR[i + (size_t)j * N];
      zc a = D1m[i] * std::conj(udv1.U[j + (size_t)i * N]);
      zc b = -D2m[i] * udv2.V[i + (size_t)j * N];
      if (first) { HLPB2[i + (size_t)(j + N) * N2] = a; HLPB2[(i + N) + (size_t)j * N2] = b; }
      else { HLPB2[i + (size_t)(j + N) * N2] = b; HLPB2[(i + N) + (size_t)j * N2] = a; }
    }
  for (int j = 0; j < N2; ++j) for (int i = 0; i < N2; ++i) HLPB1[i + (size_t)j * N2] = std::conj(HLPB2[j + (size_t)i * N2]);
  qdrp(N2, HLPB1.data(), D3.data(), ipvt.data(), tau);
  if (first) {
    solve_extended(N, HLPB2.data(), V1INV.data(), MYU2.data(), HLPB1.data(), D3.data(), tau, ipvt.data());
    get_blocks(N, HLPB2.data(), GR00, GR0T, GRT0, GRTT);
  } else {
    solve_extended(N, HLPB2.data(), MYU2.data(), V1INV.data(), HLPB1.data(), D3.data(), tau, ipvt.data());
    get_blocks(N, HLPB2.data(), GRTT, GRT0, GR0T, GR00);
  }
}

// ---------------------------------------------------------------------------
// C API
// ---------------------------------------------------------------------------
extern "C" {

struct oracle_stats {
  int64_t n_prop, n_acc, n_prop_eff, n_acc_eff;
  int64_t ncg; double xmeanG_sum, xmaxG, xmaxP;
  int64_t ncg_tau; double xmean_tau_sum, xmax_tau;
};

void* oracle_create(int N, int F, int NSUN, int M, int L, int Nwrap, int ltau) {
  if (!LA.h) return nullptr;
  Oracle* o = new Oracle();
  o->N = N; o->F = F; o->NSUN = NSUN; o->M = M; o->L = L; o->Nwrap = Nwrap; o->ltau = ltau;
  o->Nstm = (L % Nwrap == 0) ? L / Nwrap : L / Nwrap + 1;
  o->stab_nt.resize(o->Nstm + 1);
  o->stab_nt[0] = 0;
  for (int n = 1; n < o->Nstm; ++n) o->stab_nt[n] = Nwrap * n;
  o->stab_nt[o->Nstm] = L;
  o->f.assign((size_t)M * L, 1);
  o->G.assign((size_t)F * N * N, 0.0);
  o->udvl.resize(F); o->udvr.resize(F); o->udvst.resize((size_t)o->Nstm * F);
  for (auto& u : o->udvl) u.alloc(N);
  for (auto& u : o->udvr) u.alloc(N);
  for (auto& u : o->udvst) u.alloc(N);
  o->phase = 1.0;
  std::memset(&o->st, 0, sizeof(o->st));
  return o;
}

void oracle_destroy(void* h) { delete (Oracle*)h; }

int oracle_set_model(void* h, const double* expT, const double* expTinv, const int* op_n, const int* op_nz,
                     const int* op_diag, const int* op_type, const int* op_P, const zc* op_g, const zc* op_alpha,
                     const double* op_E, const zc* op_U, const zc* op_Eexp, const zc* op_Mexp) {
  Oracle& o = *(Oracle*)h;
  size_t K = (size_t)o.F * o.M, NN = (size_t)o.N * o.N;
  o.expT.assign(expT, expT + o.F * NN);
  o.expTinv.assign(expTinv, expTinv + o.F * NN);
  o.op_n.assign(op_n, op_n + K); o.op_nz.assign(op_nz, op_nz + K); o.op_diag.assign(op_diag, op_diag + K);
  o.op_type.assign(op_type, op_type + K); o.op_P.assign(op_P, op_P + 2 * K);
  o.op_g.assign(op_g, op_g + K); o.op_alpha.assign(op_alpha, op_alpha + K);
  o.op_E.assign(op_E, op_E + 2 * K); o.op_U.assign(op_U, op_U + 4 * K);
  o.op_Eexp.assign(op_Eexp, op_Eexp + 10 * K); o.op_Mexp.assign(op_Mexp, op_Mexp + 20 * K);
  for (size_t k = 0; k < K; ++k)
    for (int a = 0; a < o.op_n[k]; ++a)
      if (o.op_P[2 * k + a] < 0 || o.op_P[2 * k + a] >= o.N) return 6;  // ERROR_HAMILTONIAN
  return 0;
}

// Checkerboard hopping: ncheck bond operators per flavour (P 0-based, [F][ncheck][2]; mat, inv
// [F][ncheck][4] column-major 2 x 2), replacing the dense exponentials; ncheck = 0 restores them.
int oracle_set_checkerboard(void* h, int ncheck, const int* P, const double* mat, const double* inv) {
  Oracle& o = *(Oracle*)h;
  o.ncheck = ncheck;
  o.cb_P.assign(P, P + 2 * (size_t)o.F * ncheck);
  o.cb_mat.assign(mat, mat + 4 * (size_t)o.F * ncheck);
  o.cb_inv.assign(inv, inv + 4 * (size_t)o.F * ncheck);
  for (int v : o.cb_P)
    if (v < 0 || v >= o.N) return 6;  // ERROR_HAMILTONIAN
  return 0;
}

int oracle_set_fields(void* h, const int8_t* f) {
  Oracle& o = *(Oracle*)h;
  for (size_t i = 0; i < (size_t)o.M * o.L; ++i) {
    int v = f[i];
    if (v != 1 && v != -1 && v != 2 && v != -2) return 5;  // ERROR_FIELDS
  }
  o.f.assign(f, f + (size_t)o.M * o.L);
  return 0;
}
int oracle_get_fields(void* h, int8_t* f) {
  Oracle& o = *(Oracle*)h;
  std::memcpy(f, o.f.data(), (size_t)o.M * o.L);
  return 0;
}
int oracle_get_green(void* h, zc* G) {
  Oracle& o = *(Oracle*)h;
  std::memcpy(G, o.G.data(), o.G.size() * sizeof(zc));
  return 0;
}
int oracle_set_green(void* h, const zc* G) {
  Oracle& o = *(Oracle*)h;
  std::memcpy(o.G.data(), G, o.G.size() * sizeof(zc));
  return 0;
}
void oracle_get_stats(void* h, oracle_stats* s) { std::memcpy(s, &((Oracle*)h)->st, sizeof(oracle_stats)); }
void oracle_reset_stats(void* h) { std::memset(&((Oracle*)h)->st, 0, sizeof(Stats)); }
void oracle_get_phase(void* h, zc* ph) { *ph = ((Oracle*)h)->phase; }

void oracle_set_recording(void* h, int8_t* acc, zc* ratio, zc* G, zc* Gwrap, zc* phase) {
  Oracle& o = *(Oracle*)h;
  o.rec_acc = acc; o.rec_ratio = ratio; o.rec_G = G; o.rec_Gwrap = Gwrap; o.rec_phase = phase;
  o.rec_visit = 0; o.rec_stab = 0;
}

// Init chain (main.F90:589-631)
int oracle_init_state(void* h, zc* phase_out) {
  Oracle& o = *(Oracle*)h;
  for (int nf = 0; nf < o.F; ++nf) {
    o.udvl[nf].reset(o.N, 'l');
    o.udvr[nf].reset(o.N, 'r');
    o.udvst[(size_t)(o.Nstm - 1) * o.F + nf].reset(o.N, 'l');
  }
  for (int nst = o.Nstm - 1; nst >= 1; --nst) {
    wrapul(o, o.stab_nt[nst + 1], o.stab_nt[nst], o.udvl);
    for (int nf = 0; nf < o.F; ++nf) o.udvst[(size_t)(nst - 1) * o.F + nf] = o.udvl[nf];
  }
  wrapul(o, o.stab_nt[1], 0, o.udvl);
  zc ph = 1.0;
  for (int nf = 0; nf < o.F; ++nf) {
    zc Z;
    cgr(o.N, Z, 1, o.Gf(nf), o.udvr[nf], o.udvl[nf]);
    op_phase(o, Z, nf);
    ph *= Z;
  }
  o.phase = std::pow(ph, (double)o.NSUN);
  if (phase_out) *phase_out = o.phase;
  return 0;
}

static int oracle_tau_m(Oracle& o);

// One sequential sweep (main.F90:714-887), resumable in chunks of time slices so that a
// bounded sample of sweep work can be timed.  u: 3*2*M*L draws in visit order.
// Returns 1 when the sweep (including the final stabilisation and TAU_M) is complete,
// 0 when more slices remain, or an ALF error code (>1 is returned negated).
int oracle_sweep_chunk(void* h, const double* u, int nslices) {
  Oracle& o = *(Oracle*)h;
  const size_t per_slice = (size_t)3 * o.M;
  SweepCursor& cur = o.cur;
  if (!cur.active) {
    for (int nf = 0; nf < o.F; ++nf) o.udvr[nf].reset(o.N, 'r');
    cur.active = true; cur.phase = 0; cur.ntau = 0; cur.NST = 1;
  }
  int done = 0;
  while (done < nslices && cur.phase < 2) {
    if (cur.phase == 0) {
      const int ntau = cur.ntau, ntau1 = ntau + 1;
      wrapgrup(o, ntau, u + (size_t)ntau * per_slice);
      if (ntau1 == o.stab_nt[cur.NST]) {
        wrapur(o, o.stab_nt[cur.NST - 1], ntau1, o.udvr);
        for (int nf = 0; nf < o.F; ++nf) {
          o.udvl[nf] = o.udvst[(size_t)(cur.NST - 1) * o.F + nf];
          o.udvst[(size_t)(cur.NST - 1) * o.F + nf] = o.udvr[nf];
        }
        int e = stabilise(o, (ntau1 > o.L / 2) ? 2 : 1);
        if (e) { cur.active = false; return -e; }
        cur.NST++;
      }
      if (o.eq_cb) o.eq_cb(o.eq_ctx, ntau1, o.G.data(), o.phase);  // LOBS_ST = 1, LOBS_EN = Ltrot
      obs_scal(o);
      cur.ntau++;
      if (cur.ntau == o.L) {
        for (int nf = 0; nf < o.F; ++nf) o.udvl[nf].reset(o.N, 'l');
        cur.phase = 1; cur.ntau = o.L; cur.NST = o.Nstm - 1;
      }
    } else {
      const int ntau = cur.ntau, ntau1 = ntau - 1;
      wrapgrdo(o, ntau, u + (size_t)o.L * per_slice + (size_t)(o.L - ntau) * per_slice);
      if (o.eq_cb && ntau1 >= 1) o.eq_cb(o.eq_ctx, ntau1, o.G.data(), o.phase);
      if (ntau1 >= 1) obs_scal(o);
      if (cur.NST >= 1 && o.stab_nt[cur.NST] == ntau1 && ntau1 != 0) {
        wrapul(o, o.stab_nt[cur.NST + 1], ntau1, o.udvl);
        for (int nf = 0; nf < o.F; ++nf) {
          o.udvr[nf] = o.udvst[(size_t)(cur.NST - 1) * o.F + nf];
          o.udvst[(size_t)(cur.NST - 1) * o.F + nf] = o.udvl[nf];
        }
        int e = stabilise(o, (ntau1 > o.L / 2) ? 2 : 1);
        if (e) { cur.active = false; return -e; }
        cur.NST--;
      }
      cur.ntau--;
      if (cur.ntau == 0) cur.phase = 2;
    }
    ++done;
  }
  if (cur.phase < 2) return 0;
  wrapul(o, o.stab_nt[1], o.stab_nt[0], o.udvl);
  for (int nf = 0; nf < o.F; ++nf) o.udvr[nf].reset(o.N, 'r');
  cur.active = false;
  int e = stabilise(o, 1);
  if (e) return -e;
  for (int nf = 0; nf < o.F; ++nf) o.udvst[(size_t)(o.Nstm - 1) * o.F + nf].reset(o.N, 'l');
  if (o.ltau == 1) {
    e = oracle_tau_m(o);
    if (e) return -e;
  }
  return 1;
}

int oracle_sweep(void* h, const double* u) {
  int r;
  while ((r = oracle_sweep_chunk(h, u, 1 << 30)) == 0) {
  }
  return r == 1 ? 0 : -r;
}

// Component entry points for unit tests -------------------------------------------------------
int oracle_cgr(int N, int nvar, const zc* UR, const zc* DR, const zc* VR, const zc* UL, const zc* DL,
               const zc* VL, zc* G, zc* phase) {
  UDV ur, ul;
  ur.U.assign(UR, UR + (size_t)N * N); ur.V.assign(VR, VR + (size_t)N * N); ur.D.assign(DR, DR + N); ur.side = 'r';
  ul.U.assign(UL, UL + (size_t)N * N); ul.V.assign(VL, VL + (size_t)N * N); ul.D.assign(DL, DL + N); ul.side = 'l';
  cgr(N, *phase, nvar, G, ur, ul);
  return 0;
}
int oracle_decompose(int N, char side, zc* U, zc* D, zc* V) {
  UDV s;
  s.U.assign(U, U + (size_t)N * N); s.V.assign(V, V + (size_t)N * N); s.D.assign(D, D + N); s.side = side;
  decompose(N, s);
  std::memcpy(U, s.U.data(), (size_t)N * N * sizeof(zc));
  std::memcpy(V, s.V.data(), (size_t)N * N * sizeof(zc));
  std::memcpy(D, s.D.data(), (size_t)N * sizeof(zc));
  return 0;
}
// The case of the reference's solve_extended_System test (testsuite/Prog.tests/
// 17-solve-extended-system.F90): QDRP of the 2N x 2N input (in place: R above with rows
// normalised by D3, reflectors below), U3 = Q (ZUNGQR), V3 = upper(R) with its columns moved
// back by the pivots (ZLAPMT backward), and HLP = solve_extended_System(UCT, VINV, ...).
int oracle_solve_extended_case(int N, zc* input, const zc* UCT, const zc* VINV, zc* HLP, zc* U3, zc* V3, zc* D3) {
  const int N2 = 2 * N;
  vector<int> ipvt(N2);
  vector<zc> tau;
  qdrp(N2, input, D3, ipvt.data(), tau);
  std::memcpy(U3, input, (size_t)N2 * N2 * sizeof(zc));
  int info = 0, lw = -1;
  zc wq;
  LA.zungqr(&N2, &N2, &N2, U3, &N2, tau.data(), &wq, &lw, &info);
  lw = (int)std::real(wq);
  vector<zc> work(std::max(lw, 1));
  LA.zungqr(&N2, &N2, &N2, U3, &N2, tau.data(), work.data(), &lw, &info);
  for (int j = 0; j < N2; ++j)  // column j of upper(R) goes to column ipvt[j] - 1
    for (int i = 0; i < N2; ++i)
      V3[i + (size_t)(ipvt[j] - 1) * N2] = (i <= j) ? input[i + (size_t)j * N2] : zc(0.0);
  solve_extended(N, HLP, UCT, VINV, input, D3, tau, ipvt.data());
  return info;
}
// One WRAPGRUP / WRAPGRDO on the handle's G (u: 3*M draws)
int oracle_wrapgrup(void* h, int ntau, const double* u) { wrapgrup(*(Oracle*)h, ntau, u); return 0; }
int oracle_wrapgrdo(void* h, int ntau, const double* u) { wrapgrdo(*(Oracle*)h, ntau, u); return 0; }

void oracle_set_tau_callback(void* h, void (*cb)(void*, int, const zc*, const zc*, const zc*, const zc*, zc),
                             void* ctx) {
  Oracle& o = *(Oracle*)h;
  o.tau_cb = cb; o.tau_ctx = ctx;
}
void oracle_set_eq_callback(void* h, void (*cb)(void*, int, const zc*, zc), void* ctx) {
  Oracle& o = *(Oracle*)h;
  o.eq_cb = cb; o.eq_ctx = ctx;
}
// H: F x N x N real column-major (NULL: off), U: N.  Accumulators are cleared.
void oracle_set_scalar_obs(void* h, const double* H, const double* U) {
  Oracle& o = *(Oracle*)h;
  const size_t NN = (size_t)o.N * o.N;
  if (H) { o.obsH.assign(H, H + o.F * NN); o.obsU.assign(U, U + o.N); }
  else { o.obsH.clear(); o.obsU.clear(); }
  for (auto& z : o.obs_sum) z = 0.0;
  o.obs_sign = 0.0; o.obs_count = 0;
}
// out: Kin, Pot, Part, Ener as (re, im), sum of ZS, count; then cleared when reset != 0.
void oracle_get_scalar_obs(void* h, double* out, int reset) {
  Oracle& o = *(Oracle*)h;
  for (int k = 0; k < 4; ++k) { out[2 * k] = o.obs_sum[k].real(); out[2 * k + 1] = o.obs_sum[k].imag(); }
  out[8] = o.obs_sign; out[9] = (double)o.obs_count;
  if (reset) { for (auto& z : o.obs_sum) z = 0.0; o.obs_sign = 0.0; o.obs_count = 0; }
}

}  // extern "C"

// TAU_M (Prog/tau_m_mod.F90:56-211), finite temperature, no projector.
static int oracle_tau_m(Oracle& o) {
  int N = o.N, F = o.F;
  size_t NN = (size_t)N * N;
  vector<zc> G00(o.G), GT0(o.G), GTT(o.G), G0T((size_t)F * NN);
  for (int nf = 0; nf < F; ++nf)
    for (int j = 0; j < N; ++j)
      for (int i = 0; i < N; ++i) {
        zc g = o.G[(size_t)nf * NN + i + (size_t)j * N];
        G0T[(size_t)nf * NN + i + (size_t)j * N] = -((i == j ? 1.0 : 0.0) - g);
      }
  if (o.tau_cb) o.tau_cb(o.tau_ctx, 0, GT0.data(), G0T.data(), G00.data(), GTT.data(), o.phase);
  vector<UDV> udvr(F);
  for (int nf = 0; nf < F; ++nf) { udvr[nf].alloc(N); udvr[nf].reset(N, 'r'); }
  int NST = 1;
  for (int NT = 0; NT < o.L; ++NT) {
    int NT1 = NT + 1;
    for (int nf = 0; nf < F; ++nf) {
      propr(o, GT0.data() + (size_t)nf * NN, NT1, nf);
      proprm1(o, G0T.data() + (size_t)nf * NN, NT1, nf);
      proprm1(o, GTT.data() + (size_t)nf * NN, NT1, nf);
      propr(o, GTT.data() + (size_t)nf * NN, NT1, nf);
    }
    if (o.tau_cb) o.tau_cb(o.tau_ctx, NT1, GT0.data(), G0T.data(), G00.data(), GTT.data(), o.phase);
    if (NST <= o.Nstm && NT1 == o.stab_nt[NST]) {
      wrapur(o, o.stab_nt[NST - 1], o.stab_nt[NST], udvr);
      vector<zc> H1(NN), H2(NN), H3(NN), H4(NN);
      for (int nf = 0; nf < F; ++nf) {
        cgr2_2(N, H1.data(), H2.data(), H3.data(), H4.data(), udvr[nf], o.udvst[(size_t)(NST - 1) * F + nf]);
        double xmax, xmean;
        zc* gt0 = GT0.data() + (size_t)nf * NN; zc* g00 = G00.data() + (size_t)nf * NN;
        zc* gtt = GTT.data() + (size_t)nf * NN; zc* g0t = G0T.data() + (size_t)nf * NN;
        compare(N, H1.data(), gt0, xmax, xmean); o.st.ncg_tau++; o.st.xmax_tau = std::max(o.st.xmax_tau, xmax); o.st.xmean_tau_sum += xmean;
        compare(N, H2.data(), g00, xmax, xmean); o.st.ncg_tau++; o.st.xmax_tau = std::max(o.st.xmax_tau, xmax); o.st.xmean_tau_sum += xmean;
        compare(N, H3.data(), gtt, xmax, xmean); o.st.ncg_tau++; o.st.xmax_tau = std::max(o.st.xmax_tau, xmax); o.st.xmean_tau_sum += xmean;
        compare(N, H4.data(), g0t, xmax, xmean); o.st.ncg_tau++; o.st.xmax_tau = std::max(o.st.xmax_tau, xmax); o.st.xmean_tau_sum += xmean;
        std::memcpy(gt0, H1.data(), NN * sizeof(zc)); std::memcpy(g00, H2.data(), NN * sizeof(zc));
        std::memcpy(gtt, H3.data(), NN * sizeof(zc)); std::memcpy(g0t, H4.data(), NN * sizeof(zc));
      }
      NST++;
    }
  }
  return 0;
}
