/*
 * alfgpu -- GB300-native finite-temperature AFQMC sweep (ALF drop-in).
 *
 * C ABI of the GPU library.  All matrices are complex128 stored Fortran-style
 * (column-major, interleaved real/imaginary doubles), i.e. the memory layout of
 * ALF's `Complex(Kind=Kind(0.d0)) :: GR(Ndim,Ndim,N_FL)`.  Every entry point
 * returns an int status from ALF's runtime_error_mod enumeration
 * (Libraries/Modules/runtime_error_mod.F90:57-66) or one of the library codes
 * >= 100; the library never aborts the process and never traps on the device.
 *
 * One handle holds n_chains independent Markov chains that share Ndim, N_FL,
 * N_SUN, the number of vertices and Ltrot; each chain has its own vertex tables
 * (so U may differ per chain), its own fields, G, UDV stack and draw stream.
 * All sweep state stays resident on the GPU between calls.
 *
 * Replaced reference interfaces (paths inside the ALF tree):
 *   alfgpu_init_state  <- Prog/main.F90:589-631 (WRAPUL chain + CGR + Op_phase)
 *   alfgpu_sweep       <- Prog/main.F90:714-887 (the `If (get_sequential())` block:
 *                         WRAPGRUP Prog/Wrapgr_mod.F90:81, WRAPGRDO :160,
 *                         WRAPUR Prog/wrapur_mod.F90:37, WRAPUL Prog/wrapul_mod.F90:36,
 *                         CGR Prog/cgr1_mod.F90:36, Upgrade2 Prog/upgrade_mod.F90:105,
 *                         and TAU_M Prog/tau_m_mod.F90:56 when ltau = 1)
 *   alfgpu_cgr         <- CGR(PHASE, NVAR, GRUP, udvr, udvl), Prog/cgr1_mod.F90:36
 *   alfgpu_decompose   <- decompose_UDV_state, Prog/udv_state_mod.F90:448
 */
#ifndef ALFGPU_H
#define ALFGPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes: 0..9 mirror runtime_error_mod.F90:57-66. */
enum {
  ALFGPU_ERROR_NONE = 0,
  ALFGPU_ERROR_GENERIC = 1,
  ALFGPU_ERROR_FILE_NOT_FOUND = 2,
  ALFGPU_ERROR_UNSTABLE_MATRIX = 3, /* Precision Green > 10 (control_mod.F90:267-294) */
  ALFGPU_ERROR_MISSING_OBS = 4,
  ALFGPU_ERROR_FIELDS = 5,          /* field value outside {+-1, +-2} */
  ALFGPU_ERROR_HAMILTONIAN = 6,     /* invalid operator tables */
  ALFGPU_ERROR_GLOBAL_UPDATES = 7,
  ALFGPU_ERROR_MAXENT = 8,
  ALFGPU_ERROR_RUNNING_FILE_FOUND = 9,
  ALFGPU_ERROR_CUDA = 100,          /* a CUDA runtime call failed */
  ALFGPU_ERROR_ARGUMENT = 101,      /* bad pointer / size / index */
  ALFGPU_ERROR_UNSUPPORTED = 102,   /* model feature not implemented on the GPU */
  ALFGPU_ERROR_NAN = 103,           /* NaN in G (control_mod.F90:219-263 aborts with ERROR_GENERIC) */
  ALFGPU_ERROR_TIMEOUT = 104,       /* a bounded device-side wait gave up */
  ALFGPU_ERROR_SIZE = 105           /* size above a fixed maximum (see alfgpu_decompose_noalloc) */
};

/* Precision forms.  FP64: complex128 throughout; every product on the FP64 pipes
 * (mma.sync m8n8k4 f64), the per-visit Metropolis chain, QRs, solves and phases in FP64.
 * MIXED: G and all state stay complex128.  By default the G wraps through exp(-dtau T),
 * the UDV propagation products and the stabilisation's complex products (CGR's
 * U_R^H U_L and D_R V_R V_L D_L, the products with Q, decompose's R P V) run on the BF16
 * tensor cores (tcgen05) as digit-sliced products exact to ~2^-54 of the row / column
 * scales; on grids of several chains the delayed-update flushes and the explicit Q do
 * too (one chain keeps the double-float flush and the FP64 explicit Q).  The per-visit
 * Metropolis ratio, its accept test, the phase update and the block-submatrix updates
 * run in double-float (FP32 hi/lo pairs, ~2^-46 relative rounding per operation) on the
 * FP32 pipes.  The pivoted QRs, triangular solves, determinant phases of CGR / CGR2_2
 * and Precision Green stay FP64 arithmetic.  ALFGPU_FLAG_NO_TENSOR_GEMM replaces the
 * tensor-core products of the wraps and flushes by double-float GEMMs;
 * ALFGPU_FLAG_DF_PROPAGATION runs the UDV propagation products in double-float (the
 * product of Nwrap slices is ill-conditioned, 1e5-1e10 at beta = 10, so this is only
 * usable for small beta / Nwrap). */
enum { ALFGPU_PRECISION_FP64 = 0, ALFGPU_PRECISION_MIXED = 1 };
enum { ALFGPU_FLAG_DF_PROPAGATION = 1 };
/* Column pivoting of the stabilisation QRs.  Default, in both precision forms: ZGEQP3's
 * dynamic pivoting with norm downdates (Prog/QDRP_decompose_mod.F90:60-101, the
 * reference's default branch) on one thread-block cluster per matrix, for every QR.
 * ALFGPU_FLAG_NORM_PIVOT_CGR / _DECOMPOSE instead order the columns of that call site's
 * QR once by their norms and factor them with the blocked unpivoted QR (the pivoting of
 * ALF's STABLOG branch, Prog/udv_state_mod.F90:503-542), whose trailing work runs on all
 * SMs; ALFGPU_FLAG_EXACT_QRP forces ZGEQP3 pivoting everywhere.  Measured on the 16x16
 * beta = 10 Hubbard model: norm pivoting in decompose raises Precision Green from ~7e-7
 * to 3e-4 (one chain); in CGR, over 16 chains x 7 sweeps of the mixed form, the largest
 * Precision Green rises from 8.7e-6 to 1.3e-5 and the sweep is slower (15.2 vs 14.8
 * sweeps/s), while G at every stabilisation point still agrees with the ZGEQP3 oracle to
 * 1e-10.  ZGEQP3 pivoting is always used for Ndim > 512. */
enum { ALFGPU_FLAG_EXACT_QRP = 2, ALFGPU_FLAG_NORM_PIVOT_CGR = 4, ALFGPU_FLAG_NORM_PIVOT_DECOMPOSE = 8,
       ALFGPU_FLAG_NORM_PIVOT = 12 };
/* Mixed form only, opt-in: run parts of the stabilisation in double-float instead of
 * FP64.  _QR: the pivoted QR and explicit Q of decompose_UDV_state (the columns are
 * factored unscaled, exact in exponent range); _GEMM: the UDV propagation, decompose
 * and CGR products.  Measured on the 16x16 beta = 10 Hubbard chain, Precision Green
 * rises from 2.5e-6 (FP64) to 7.9e-6 (_QR) and 2.1e-5 (both): double-float keeps 48
 * of FP64's 53 mantissa bits, and the UDV products amplify rounding. */
enum { ALFGPU_FLAG_DF_STAB_QR = 16, ALFGPU_FLAG_DF_STAB_GEMM = 32, ALFGPU_FLAG_DF_STAB = 48 };
/* alfgpu_sweep captures its launch sequence into a CUDA graph on first use (one per
 * draw source) and replays it; sweeps with a callback, recording, profiling or TAU_M
 * use the stream path.  ALFGPU_FLAG_NO_GRAPH always uses the stream path. */
enum { ALFGPU_FLAG_NO_GRAPH = 64 };
/* Mixed form: the G wraps and delayed-update flushes run as digit-sliced BF16 products on
 * the tensor cores (tcgen05), exact to ~2^-54 like FP64 (N_dim <= 448); this flag selects
 * the double-float GEMMs on the FP32 pipes instead. */
enum { ALFGPU_FLAG_NO_TENSOR_GEMM = 128 };
/* Mixed form: the complex products inside the stabilisation (CGR's U_R^H U_L and
 * D_R V_R V_L D_L, the products with Q and the pivot permutations, decompose's R P V) run on
 * the same FP64-accurate tensor-core GEMM by default; this flag keeps them on the FP64 GEMM
 * (the pivoted QR, triangular solves and phases are FP64 arithmetic either way). */
enum { ALFGPU_FLAG_FP64_STAB_GEMM = 256 };
/* Mixed form: the tensor-core choices made for batched grids (32-wide tiles, the flush and
 * the explicit Q on the tensor cores) also for a grid that does not fill the GPU (by
 * default one chain keeps 16-wide tiles and the double-float flush / FP64 explicit Q,
 * measured faster there). */
enum { ALFGPU_FLAG_TENSOR_WIDE = 512 };
/* The exact pivoted QR (ZGEQP3 on one thread-block cluster per matrix) takes clusters of half
 * the default size when the full-size clusters of a batched launch would put more than two
 * CTAs on every SM; these flags force the half-size or the full-size cluster. */
enum { ALFGPU_FLAG_QR_HALF_CLUSTER = 1024, ALFGPU_FLAG_QR_FULL_CLUSTER = 2048 };
/* Mixed form, grids of several chains: the delayed-update flush G -= X Y on the double-float
 * GEMM, whose loop stops at the block's accepted count, instead of the tensor-core GEMM
 * (K padded to 64, digit-sliced). */
enum { ALFGPU_FLAG_DF_FLUSH = 4096 };
/* The exact pivoted QR keeps each CTA's rows in a global (L2-resident) workspace even where
 * they fit in shared memory.  A CTA then needs little shared memory, so several clusters share
 * an SM; by default this layout is taken when it needs fewer waves of clusters than rows in
 * shared memory (batched grids), and this flag takes it always. */
enum { ALFGPU_FLAG_QR_GLOBAL_ROWS = 8192 };
/* alfgpu_sweep runs a delayed-update block's Metropolis visits on a second stream while the
 * previous block's flush runs (the block's submatrix is staged from a snapshot of G and the
 * flush operands; models with vector vertices and profiled sweeps keep the serial order).
 * This flag keeps the serial order always. */
enum { ALFGPU_FLAG_NO_OVERLAP = 16384 };
/* Mixed form, grids of several chains: the K = 64 tensor-core products (delayed-update flush,
 * compact-WY update of the explicit Q) run on 16-wide tiles sized so that two of their CTAs and
 * one k_update CTA share an SM (the next block's visits overlap the flush).  This flag keeps the
 * 32-wide tiles of one CTA per SM (and the serial order of visits and flush). */
enum { ALFGPU_FLAG_OZ_FLUSH_SINGLE = 32768 };
/* Mixed form: the per-visit Metropolis arithmetic, the block-submatrix updates, Gamma^-1 and
 * the flush operand Y in FP64 (k_update<ArD>) instead of double-float. */
enum { ALFGPU_FLAG_FP64_VISITS = 65536 };
/* Mixed form: the K = N_dim tensor-core products (G wraps, UDV propagation, stabilisation
 * products) on 16-wide tiles with the deeper A ring of one-chain grids, also on batched grids. */
enum { ALFGPU_FLAG_OZ_DEEP_RING = 131072 };
/* Mixed form, grids of several chains: the K = 64 tensor-core products as persistent CTAs, one
 * per SM, each over a contiguous range of output tiles whose A digit slices stay in shared
 * memory from one tile to the next (no overlap of the visits with the flush). */
enum { ALFGPU_FLAG_OZ_FLUSH_RESIDENT = 262144 };
/* The exact pivoted QR applies each step's reflector and forms the next step's partial sums in
 * two passes over the rows (by default one pass does both, the next pivot chosen first). */
enum { ALFGPU_FLAG_QR_TWO_PASS = 524288 };

/* dims.reserved[1] / dims.reserved[2] (mixed form, tensor-core products only): target bits of
 * the digit-sliced products of the G wraps and TAU_M's propagation (reserved[1]) and of the
 * UDV propagation (reserved[2]); 0 keeps the full count (~54 bits, FP64-class).  The digits
 * are b bits wide (b = 7 for N_dim <= 128, 6 up to 448, 5 beyond), so a target rounds up to whole
 * digits; S digits cost (S + 1)(S + 2)/2 - 2 BF16 products per product (53 for S = 9, 43
 * for S = 8) and bound the error by 2^-(b S) of the row / column scales. */
enum { ALFGPU_DIMS_WRAP_BITS = 1, ALFGPU_DIMS_PROPAGATE_BITS = 2 };  /* indices into dims.reserved */

typedef struct alfgpu_s alfgpu_t;

typedef struct {
  int32_t ndim;      /* Ndim */
  int32_t n_fl;      /* N_FL (= N_FL_eff; flavour reconstruction is not used) */
  int32_t n_sun;     /* N_SUN after the model's own adjustment */
  int32_t n_op;      /* Size(Op_V,1): vertices per time slice */
  int32_t ltrot;     /* Ltrot */
  int32_t nwrap;     /* Nwrap; Stab_nt follows main.F90:446-457 */
  int32_t n_chains;  /* independent Markov chains in this handle */
  int32_t precision; /* ALFGPU_PRECISION_FP64 or ALFGPU_PRECISION_MIXED */
  int32_t delay_k;   /* vertex visits per delayed-update block (0: library default) */
  int32_t ltau;      /* 1: time-displaced Green functions (TAU_M) after every sweep */
  int32_t device;    /* CUDA device ordinal */
  int32_t reserved[5];
} alfgpu_dims;

/* Interaction vertices Op_V(n,nf) after Op_set (Prog/Operator_mod.F90:259-472),
 * struct-of-arrays with index k = nf*n_op + n.  Complex arrays are interleaved.
 *   op_n[k]      Op%N (1 or 2 sites)          op_nz[k]   Op%N_non_zero
 *   op_diag[k]   Op%diag                       op_type[k] Op%type (1 or 2)
 *   op_P[2k+a]   Op%P(a+1) - 1 (0-based site)  op_g[k], op_alpha[k]   complex
 *   op_E[2k+m]   Op%E(m+1)                     op_U[k]    2x2 column-major
 *   op_Eexp[k]   [m][s+2] = E_exp(m+1, s)      op_Mexp[k] [s+2] 2x2 column-major M_exp */
typedef struct {
  const int32_t* op_n;
  const int32_t* op_nz;
  const int32_t* op_diag;
  const int32_t* op_type;
  const int32_t* op_P;
  const double* op_g;
  const double* op_alpha;
  const double* op_E;
  const double* op_U;
  const double* op_Eexp;
  const double* op_Mexp;
} alfgpu_vertices;

typedef struct {
  int64_t n_prop, n_acc;          /* Control_upgrade counters (upgrade_mod.F90:295-298) */
  int64_t n_prop_eff, n_acc_eff;  /* Control_upgrade_eff */
  int64_t ncg;                    /* number of Precision Green comparisons */
  double xmeanG_sum, xmaxG;       /* Control_PrecisionG: sum of mean, max |G_wrap - G_fresh| */
  double xmaxP;                   /* Control_PrecisionP: max |phase_wrap - phase_fresh| */
  int64_t ncg_tau;
  double xmean_tau_sum, xmax_tau; /* Control_Precision_tau */
  int64_t sweeps;
} alfgpu_stats;

/* Observable callback: the Fortran side's ham%Obser (kind 0, G = GR(N,N,N_FL)) or
 * ham%ObserT (kind 1, G = [GT0, G0T, G00, GTT] each N x N x N_FL).  Buffers are
 * library-owned pinned memory, valid only during the call. */
typedef void (*alfgpu_obs_cb)(void* ctx, int32_t chain, int32_t ntau, int32_t kind, const double* G,
                              const double* phase);

/* Handle lifetime. */
int alfgpu_create(alfgpu_t** h, const alfgpu_dims* dims);
void alfgpu_destroy(alfgpu_t* h);
const char* alfgpu_error_string(int code);

/* Model upload.  expT / expTinv are the real `mat` / `invmat` of RealExpOpT
 * (Prog/OpTTypes_mod.F90:92-133), n_fl x Ndim x Ndim column-major, shared by all
 * chains.  Vertex tables are per chain (chain = -1 uploads the same tables to all). */
int alfgpu_upload_hopping(alfgpu_t* h, const double* expT, const double* expTinv);
/* Checkerboard hopping (Checkerboard = .T.; Op_T built by Predefined_Hop_mod.F90:1773-1839 as
 * one two-site operator per bond): ncheck bond operators per flavour in Op_T order, P
 * [n_fl][ncheck][2] 0-based sites, mat = exp(g O) and inv = exp(-g O) [n_fl][ncheck][4]
 * real column-major 2 x 2, grouped into nfam families of disjoint bonds (operators
 * fam[q] .. fam[q+1]-1, fam[0] = 0, fam[nfam] = ncheck).  Every hopping product of the sweep,
 * the UDV propagation and TAU_M then applies the bonds in the order of the Hop_mod routine it
 * replaces (Hop_mod.F90:143-250: B_T = E_1 ... E_ncheck), one launch per family, in place of
 * the dense exp(-dtau T) products of alfgpu_upload_hopping; ncheck = 0 returns to those.  Not
 * for models with two-site vertices (ALFGPU_ERROR_UNSUPPORTED). */
int alfgpu_upload_checkerboard(alfgpu_t* h, int32_t ncheck, int32_t nfam, const int32_t* fam, const int32_t* P,
                               const double* mat, const double* inv);
int alfgpu_upload_vertices(alfgpu_t* h, int32_t chain, const alfgpu_vertices* v);

/* Fields nsigma%f(n, nt): int8 values in {+-1, +-2}, Ltrot x n_op (n fastest). */
int alfgpu_set_fields(alfgpu_t* h, int32_t chain, const int8_t* f);
/* Same, from ALF's complex storage (real parts are the field values). */
int alfgpu_set_fields_c128(alfgpu_t* h, int32_t chain, const double* f);
int alfgpu_get_fields(alfgpu_t* h, int32_t chain, int8_t* f);

/* Per-chain draw stream used when alfgpu_sweep gets uniforms = NULL. */
int alfgpu_set_rng(alfgpu_t* h, int32_t chain, uint64_t seed, uint64_t counter);
/* Checkpoint / resume of a chain (the reference writes the fields and its generator state to
 * confout_<rank>, Fields_mod.F90:474-506, and reads them back, :750-778): the draw stream's
 * key and next counter.  With alfgpu_get_fields / alfgpu_set_fields and alfgpu_init_state
 * (G is rebuilt from the fields, as on the reference's restart) a chain resumes on the same
 * draws. */
int alfgpu_get_rng_state(alfgpu_t* h, int32_t chain, uint64_t* key, uint64_t* counter);
int alfgpu_set_rng_state(alfgpu_t* h, int32_t chain, uint64_t key, uint64_t counter);

/* Initial UDV stack and G (main.F90:589-631); phase_out: complex per chain (may be NULL). */
int alfgpu_init_state(alfgpu_t* h, double* phase_out);

/* One sequential sweep on every chain.  uniforms: host array n_chains x (6*n_op*Ltrot),
 * three draws per vertex visit in visit order (up pass nt=1..L, n=1..M; down pass
 * nt=L..1, n=M..1; slots: flip choice, T0 test, Metropolis), or NULL for the
 * device stream.  cb may be NULL (no measurements). */
int alfgpu_sweep(alfgpu_t* h, const double* uniforms, alfgpu_obs_cb cb, void* ctx);

/* One sweep on each of n handles (no counterpart in the reference, whose walkers are MPI
 * ranks): every handle's launches are issued first, each on its own stream (its captured
 * graph replays where alfgpu_sweep would replay it), then each handle is waited for and
 * checked, so handles of different N_dim / Ltrot sweep concurrently from one host thread.
 * uniforms: NULL (every handle's device stream) or n pointers as for alfgpu_sweep (a NULL
 * entry: that handle's device stream).  status[k] receives handle k's alfgpu_sweep code; the
 * return value is the first non-zero one.  No measurement callbacks: use alfgpu_sweep, or the
 * device-side observables, for measuring sweeps.  The handles may share a device or not. */
int alfgpu_sweep_many(alfgpu_t* const* hs, int32_t n, const double* const* uniforms, int32_t* status);

/* Stabilisation interval Nwrap (the reference's fixed Nwrap, main.F90:446-457): re-plans the
 * stabilisation points and grows the UDV stack as needed; G and the stack must then be
 * rebuilt from the current fields with alfgpu_init_state before the next sweep.  A driver
 * shortens Nwrap when Precision Green (alfgpu_get_stats) exceeds its bound. */
int alfgpu_set_nwrap(alfgpu_t* h, int32_t nwrap);
int alfgpu_get_nwrap(alfgpu_t* h, int32_t* nwrap);

/* Delay depth k of the delayed (block submatrix) update: at most k positions per
 * block before the rank-k flush (2..32; the default is dims.delay_k or 32).
 * alfgpu_tune_delay is the autotuner: it runs nsweeps sweeps on the device draw stream
 * (thermalisation sweeps: they advance the chains) with each k in {8, 16, 24, 32},
 * times the update and flush phases, and keeps the fastest k.  No counterpart in the
 * reference (ALF has no delayed update). */
int alfgpu_set_delay(alfgpu_t* h, int32_t k);
int alfgpu_get_delay(alfgpu_t* h, int32_t* k);
int alfgpu_tune_delay(alfgpu_t* h, int32_t nsweeps, int32_t* k_out);

/* State readback. */
int alfgpu_get_green(alfgpu_t* h, int32_t chain, double* G);  /* Ndim x Ndim x N_FL */
int alfgpu_get_phase(alfgpu_t* h, double* phase);             /* complex per chain */
int alfgpu_get_stats(alfgpu_t* h, int32_t chain, alfgpu_stats* s);
int alfgpu_reset_stats(alfgpu_t* h);

/* Parity recording (diagnostics): while enabled, every vertex visit's ratio and
 * accept bit, and G and the phase at every stabilisation point are kept on the
 * device for the next sweep; alfgpu_get_record copies them out for one chain.
 * Sizes per sweep: visits = 2*n_op*Ltrot, points = 2*Nstm with Nstm = ceil(Ltrot / Nwrap)
 * for the handle's CURRENT Nwrap (alfgpu_get_nwrap; alfgpu_set_nwrap changes it): the
 * caller's buffers must hold that many points. */
int alfgpu_set_recording(alfgpu_t* h, int32_t enable);
int alfgpu_get_record(alfgpu_t* h, int32_t chain, int8_t* acc, double* ratio, double* G_fresh,
                      double* G_wrapped, double* phase);

/* Stream the library launches on (a cudaStream_t), for callers that overlap work.  Work the
 * sweep puts on its second stream (see ALFGPU_FLAG_NO_OVERLAP) is joined back into this stream
 * before the sweep's next launch on it, so an event recorded or a synchronisation on this stream
 * after alfgpu_sweep covers the whole sweep. */
void* alfgpu_stream(alfgpu_t* h);

/* Phase profiling (diagnostics): while enabled, CUDA events on the library
 * stream time each group of launches by phase; alfgpu_get_profile returns the
 * accumulated milliseconds and launch-group counts per phase. */
enum {
  ALFGPU_PROF_HOP = 0,       /* exp(-dtau T) wraps of G (Wrapgr_mod.F90:110-114, 237-241) */
  ALFGPU_PROF_UPDATE = 1,    /* Metropolis blocks (Upgrade2) */
  ALFGPU_PROF_FLUSH = 2,     /* delayed-update flushes */
  ALFGPU_PROF_PROPAGATE = 3, /* UDV propagation of WRAPUR / WRAPUL */
  ALFGPU_PROF_QR = 4,        /* pivoted QR (QDRP_decompose) */
  ALFGPU_PROF_ORGQR = 5,     /* explicit Q */
  ALFGPU_PROF_SOLVE = 6,     /* triangular solves of CGR */
  ALFGPU_PROF_N = 7
};
int alfgpu_set_profiling(alfgpu_t* h, int32_t enable);
int alfgpu_get_profile(alfgpu_t* h, double* ms, int64_t* launches);
/* Number of kernel launches this handle has issued so far. */
int64_t alfgpu_launch_count(alfgpu_t* h);

/* One-shot component entry points on host buffers (allocate their own device memory). */
int alfgpu_cgr(int32_t ndim, int32_t nvar, const double* UR, const double* DR, const double* VR, const double* UL,
               const double* DL, const double* VL, double* G, double* phase);
int alfgpu_decompose(int32_t ndim, char side, double* U, double* D, double* V);

/* decompose_UDV_state on DEVICE buffers without allocating any device memory.
 * This entry point has no counterpart in the reference.  It exists for callers
 * that cannot or must not allocate: a host program whose device memory is
 * already owned by another allocator (a framework's caching pool), or one that
 * must not trigger the implicit device synchronisation of cudaMalloc/cudaFree
 * in the middle of its stream work.  The caller passes its own device
 * pointers: U (ndim x ndim complex128, column-major, in/out), D (ndim doubles,
 * in/out: the scales, real), V (ndim x ndim complex128, in/out), detU (one
 * complex128, out: det(U) after the decomposition; may be NULL) and the
 * cudaStream_t to launch on (NULL = legacy default stream).  All scratch lives
 * in one file-scope device array sized for ndim <= ALFGPU_NOALLOC_MAX_NDIM
 * (about 1.06 MiB, held by every GPU that loads the library until the process
 * exits); larger ndim returns ALFGPU_ERROR_SIZE without touching the buffers.
 * The first call on each device resolves the array's device address
 * (cudaGetSymbolAddress) with that device current, so make the first call on
 * a device before any stream capture.  That set-up is guarded: host threads may
 * make their first calls on a device at the same time.  The resolved address is
 * kept for the life of the process and is valid only as long as the device's
 * primary context: after cudaDeviceReset, or a reset of the primary context by
 * another library, this entry point must not be called again in that process.
 * Every call reuses the same array, and
 * each call writes every scratch word it later reads, so no state carries over;
 * calls that overlap on the GPU (different streams or host threads) race on
 * the shared array and must be serialised by the caller.  The call is
 * stream-ordered: results are ready when the stream reaches them. */
#define ALFGPU_NOALLOC_MAX_NDIM 256
int alfgpu_decompose_noalloc(int32_t ndim, char side, double* U, double* D, double* V, double* detU, void* stream);

/* Device-side equal-time scalar observables of the Hubbard-type models (the Obs_scal part of
 * ham%Obser, Hamiltonian_Hubbard_smod.F90:695-801; kinetic term as
 * Predefined_Hoppings_Compute_Kin, Prog/Predefined_Hop_mod.F90:1905-1959).  At every
 * ham%Obser call site of the sweep (after every slice of both passes) the library adds, per
 * chain, ZP*ZS*{Kin, Pot, Part, Ener} (complex), ZS and 1 to its accumulators, with
 * GRC(i,j) = delta_ij - G(j,i), ZP = Phase/Re(Phase), ZS = sign(Re(Phase)),
 * Kin = N_SUN sum_f sum_ij H_f(i,j) GRC_f(i,j), Pot = sum_i U_i GRC_1(i,i) GRC_dec(i,i)
 * (dec = 2 for two flavours, else 1), Part = N_SUN sum_f sum_i GRC_f(i,i), Ener = Kin + Pot.
 * H: n_fl x Ndim x Ndim real column-major (the hopping Hamiltonian Op_T%O, chemical
 * potential included), U: Ndim on-site couplings (ham_U).  H = U = NULL switches it off.
 * Not for two-site (rotated-basis) vertices (ALFGPU_ERROR_UNSUPPORTED).
 * alfgpu_get_scalar_obs: 10 doubles: Kin, Pot, Part, Ener as (re, im), sum of ZS, count;
 * a bin is the accumulators between two alfgpu_reset_scalar_obs calls. */
int alfgpu_set_scalar_obs(alfgpu_t* h, const double* H, const double* U);
int alfgpu_get_scalar_obs(alfgpu_t* h, int32_t chain, double* sums);
int alfgpu_reset_scalar_obs(alfgpu_t* h);

/* Device-side lattice-resolved observables: the predefined measurements of ham%Obser and
 * ham%ObserT (Prog/Predefined_Obs_mod.F90:137-600: N_FL = 2 Green, SpinZ, SpinXY, SpinT, Den;
 * N_FL = 1 Green, SpinZ (SpinSUN), Den), accumulated per chain on the device at every
 * measurement point of the sweep (equal time) and every slice of TAU_M (time displaced), so a
 * measuring sweep copies no Green function to the host.  The lattice: site_of[cell * norb + o]
 * = the site of orbital o of cell `cell` (ncell * norb = Ndim), jof[I * ncell + R] = the cell J
 * with imj(I, J) = R (Make_lattice's imj, Libraries/Modules/lattices_v3_mod.F90:88-336).
 * site_of = jof = NULL switches it off.  alfgpu_get_lattice_obs(kind 0: equal time, 1: time
 * displaced) returns per observable (in the order above) Obs_Latt(R, nt, no_I, no_J) as
 * [name][R][nt][no_I][no_J] complex (nt: 1 slice, or Ltrot + 1 for kind 1), Obs_Latt0 as
 * [name][no] complex, and (measurements, sum of ZS); each G contributes Phase / Re(Phase)
 * sign(Re(Phase)) times its measurement; a bin is the accumulators between two resets
 * (Print_bin_Latt divides by the count, Prog/observables_mod.F90:355-500).  No counterpart in
 * the reference's interface (the Fortran side measures on the host). */
int alfgpu_set_lattice_obs(alfgpu_t* h, int32_t ncell, int32_t norb, const int32_t* site_of, const int32_t* jof);
int alfgpu_get_lattice_obs(alfgpu_t* h, int32_t chain, int32_t kind, double* latt, double* latt0, double* count_sign);
int alfgpu_reset_lattice_obs(alfgpu_t* h);

/* The CUDA call behind the last ALFGPU_ERROR_CUDA of this handle ("file:line: CUDA error
 * string"); the pointer stays valid until the next call on the handle. */
const char* alfgpu_last_error(alfgpu_t* h);

/* C = A B for real column-major host matrices (m x k, k x n, m x n with leading
 * dimensions lda, ldb, ldc) on the tensor-core GEMM of the mixed form (k_oz_gemm,
 * digit-sliced BF16 with exact FP32 accumulation, ~2^-54 relative to the row and column
 * scales of A and B; k <= 512, else ALFGPU_ERROR_SIZE).  The kernel the G wraps use,
 * exposed for testing and for callers that want FP64-accurate products on the tensor
 * cores.  Synchronous; allocates and frees its own device buffers.  No counterpart in the
 * reference. */
int alfgpu_oz_dgemm(int32_t m, int32_t n, int32_t k, const double* A, int32_t lda, const double* B, int32_t ldb,
                    double* C, int32_t ldc, int32_t device);

#ifdef __cplusplus
}
#endif
#endif /* ALFGPU_H */
