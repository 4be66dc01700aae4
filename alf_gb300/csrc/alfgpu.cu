// alfgpu: host orchestration of the sweep and the C ABI (include/alfgpu.h).
//
// The sweep follows Prog/main.F90:714-887 step by step; every matrix product,
// Metropolis block, QR and solve is a kernel on one CUDA stream, with all state
// (G, the UDV stack, fields, phase, counters) resident on the device.  The
// launch sequence of a sweep does not depend on the data (the accepted count
// of a delayed-update block is read by the flush GEMM on the device), so a
// whole sweep can be captured once into a CUDA graph and replayed.
#include <cuda_runtime.h>

#include <cstdio>
#include <cstdlib>
#include <cmath>
#include <cstring>
#include <complex>
#include <vector>

#include "common.cuh"
#include "gemm.cuh"
#include "gemm32.cuh"
#include "qr_blocked.cuh"
#include "kernels_misc.cuh"
#include "linalg.cuh"
#include "update.cuh"
#include "tau.cuh"
#include "ozaki.cuh"
#include "obs_latt.cuh"

#include <atomic>
#include <map>
#include <mutex>
#include <utility>

namespace {

struct UDVSet {  // one UDV state for all B = C*F (chain, flavour) pairs
  zd* U = nullptr;
  zd* V = nullptr;
  double* D = nullptr;
  zd* detU = nullptr;
};

}  // namespace

struct alfgpu_s {
  alfgpu_dims d;
  int N, F, M, L, C, B, Nstm, NSUN, CL, kblk, dev;
  int mixed = 0;           // double-float G wraps and flush GEMMs on the FP32 pipes, FP64 elsewhere
  int mixed_propagate = 0; // mixed form, opt-in: UDV propagation products in double-float too
  // mixed form: G wraps and delayed-update flushes as digit-sliced BF16 tensor-core GEMMs
  // (ozaki.cuh); otherwise double-float GEMMs on the FP32 pipes
  // device-side equal-time scalar observables (alfgpu_set_scalar_obs)
  int obs_scal = 0, obs_nsun = 1;
  double *obs_HT = nullptr, *obs_trH = nullptr, *obs_U = nullptr, *obs_acc = nullptr;
  // device-side lattice-resolved observables (alfgpu_set_lattice_obs): [0] equal time, [1] TAU_M
  int obs_latt = 0, lo_ncell = 0, lo_norb = 0, lo_nnames = 0;
  int *lo_site = nullptr, *lo_jof = nullptr;
  zd *lo_acc[2] = {nullptr, nullptr}, *lo_acc0[2] = {nullptr, nullptr};
  double* lo_cnt[2] = {nullptr, nullptr};
  int oz = 0, eexp_complex = 0;
  int oz_narrow = 0;  // small grids: BN = 16 tiles; the flush keeps the double-float GEMM (measured faster there)
  int oz_stab = 0;    // the stabilisation's complex products on the tensor-core GEMM too
  zd *ozGm = nullptr, *ozTm = nullptr, *ozWm = nullptr, *ozXm = nullptr;  // compact-WY explicit Q work
  int oz_bits = 0, oz_S = 0, oz_bn = 32, oz_nst = 2, oz_Kpad = 0, oz_RpN = 0, oz_Rp2N = 0;  // wraps (K = N)
  int ozf_bits = 0, ozf_S = 0, ozf_bn = 32, ozf_nst = 2;                                   // flush (K = 2 kmax)
  int ozf_pairs = 0;  // flush tiles leave room for two flush CTAs and one k_update CTA per SM
  int ozf_grid = 0;   // CTAs of the persistent K = 64 launches (paired tiles: two per SM; resident: one)
  // digit slices used by the G wraps (and TAU_M's propagation) and by the UDV propagation: a
  // prefix of the oz_S slices (dims.reserved[1] / [2] give the target bits; default oz_S)
  int ozw_S = 0, ozp_S = 0;
  unsigned short* ozE[4] = {nullptr, nullptr, nullptr, nullptr};  // expT, expTinv as A; expT, expTinv as B
  int* ozEe[4] = {nullptr, nullptr, nullptr, nullptr};
  unsigned short *ozGA = nullptr, *ozGB = nullptr, *ozXA = nullptr, *ozYB = nullptr;
  int *ozGAe = nullptr, *ozGBe = nullptr, *ozXAe = nullptr, *ozYBe = nullptr;
  CUtensorMap tmE[4], tmGA, tmGB, tmXA, tmYB;
  int exact_qrp = 0;       // current call: ZGEQP3 column pivoting (cluster kernel), else blocked pre-pivoted QR
  int exact_dec = 0, exact_cgr = 0;  // per call site: decompose_UDV_state / CGR
  int qrr_ok = 0;                    // k_qrp_rows can be launched: rows in shared memory (1) or in qrr_ws (2)
  int CLr = 1;                       // k_qrp_rows cluster size (CL, or CL / 2 on batched grids)
  zd* qrr_ws = nullptr;              // row workspace of k_qrp_rows<ArD, true> (qrr_ok == 2)
  int qr2_mode = 0, CL2 = 1;         // CGR2_2's 2N x 2N QR: 0 k_qrp, 1 / 2 as qrr_ok; its cluster size
  zd* qr2_ws = nullptr;
  // time-displaced Green functions (ltau = 1)
  int ltau = 0;
  // CUDA graphs of the sweep: [0] device draws, [1] host draws (copied before the launch)
  int use_graph = 1;
  cudaGraphExec_t gexec[2] = {nullptr, nullptr};
  long long glaunches[2] = {0, 0};
  zd *GT0 = nullptr, *G0T = nullptr, *G00 = nullptr, *GTT = nullptr, *Hn[4] = {nullptr, nullptr, nullptr, nullptr};
  UDVSet udvr_tau;
  zd *HB1 = nullptr, *HB2 = nullptr, *HLP = nullptr, *tau2 = nullptr, *V1I = nullptr, *Qt = nullptr;
  int *jpvt2 = nullptr, *first2 = nullptr;
  double *D3 = nullptr, *vn2 = nullptr, *cmp_tau = nullptr;
  QRInfo* info2 = nullptr;
  // measurement staging (pinned host memory, allocated on first use)
  double* obs_host = nullptr;
  double* tau_host = nullptr;
  double* phase_host = nullptr;
  zd* Gq = nullptr;  // [chain][4][F][N][N] device staging of the ObserT quartet
  int df_stab = 0;                   // mixed form: stabilisation products in double-float
  int df_qr = 0;                     // mixed form: decompose QR and Q formation in double-float
  int qr_df = 0;                     // the last QR left double-float reflectors in QRdf
  zd* QRdf = nullptr;                // [B][N][N] reflectors in double-float (16-byte elements)
  std::vector<int> stab_nt;
  cudaStream_t st = nullptr;
  // second stream of the sweep: a block's Metropolis visits run on it while the previous
  // block's flush runs on st (update_slice); ev_fork: st -> st2, ev_join: st2 -> st
  cudaStream_t st2 = nullptr;
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
  int overlap = 1;
  zd *Gsnap = nullptr, *Gsub = nullptr;  // [chain][F][KMAX][KMAX] next block's submatrix
  int *posn = nullptr, *npos = nullptr;  // [chain][KMAX], [chain] next block's positions
  cudaError_t last_cuda = cudaSuccess;
  int last_line = 0;        // source line of the CUDA call that failed
  char last_msg[160] = {0};
  bool hop_ok = false, vert_ok = false, fields_ok = false, state_ok = false;
  // model
  double *expT = nullptr, *expTinv = nullptr;
  int* v_site = nullptr;
  zd *v_g = nullptr, *v_alpha = nullptr, *v_Eexp = nullptr;
  UpdTab* v_tab = nullptr;  // [chain][F*M][5][3] transition factors of every (vertex, old field, flip choice)
  int* v_site2 = nullptr;   // [chain][F*M] site of the second eigen-index (two-site vertices) or -1
  int8_t* v_nsite = nullptr;  // [chain][F*M] positions (non-zero eigenvalues) of each vertex
  std::vector<int> blk_start[2], blk_cnt[2];  // delayed-update blocks of the up / down pass (visit positions)
  std::vector<int> hv_site, hv_site2;          // flavour-0 vertex sites (host), for re-blocking
  std::vector<int8_t> hv_nsite;
  // Vector vertices (single-site vertices on a site of a rotated pair, e.g. Kondo's U_f next to
  // its J_K vertex): the slice's vertices split into phases, ranges [ph_n0, ph_n1) of vertices
  // with disjoint supports; updates run in the frame of the phase's start and each phase's
  // wraps are applied explicitly (pairblock = 1).  Without them one implicit phase whose wraps
  // are deferred into the next hopping product.
  int pairblock = 0;
  std::vector<int> ph_n0, ph_n1, ph_of;        // phases and the phase of each vertex
  std::vector<int> hv_blk2;                    // flavour-0: second site of each vertex's support or -1
  std::vector<int> blk_phase_end[2];           // per block of each pass: phase that ends with it, or -1
  int8_t* v_kind = nullptr;                    // [chain][F*M] 0 one site, 1 two diagonal positions, 2 vector
  int* v_blk2 = nullptr;                       // [chain][F*M] second site of the support or -1
  double* v_vc = nullptr;                      // [chain][F*M][2] vector coefficients (c_a, c_b)
  int* sites2_out = nullptr;                   // accepted vector positions of a block: site b, coefficients
  double* coef_out = nullptr;
  int8_t* fields_old = nullptr;                // [chain][M] the slice's fields before its updates
  // checkerboard hopping (alfgpu_upload_checkerboard): bond operators per flavour in Op_T order,
  // families of disjoint bonds; replaces the dense hopping products
  int cb = 0, cb_ncheck = 0;
  std::vector<int> cb_fam;
  int* cb_P = nullptr;
  double *cb_mat = nullptr, *cb_inv = nullptr;
  std::vector<double> h_expT, h_expTinv;      // hopping exponentials as uploaded (original basis)
  bool rot = false;                           // two-site vertices: the sweep runs in the rotated basis
  std::vector<std::pair<int, int>> rot_pairs;
  double rot_U[4] = {1.0, 0.0, 0.0, 1.0};     // shared real eigenbasis, column-major
  int* rot_dev = nullptr;                     // pairs on the device
  int *v_sptr = nullptr, *v_slist = nullptr;  // [chain][F][N+1], [chain][F][M]: vertices of each site (CSR)
  double* v_E = nullptr;
  int8_t* v_type = nullptr;
  int8_t* fields = nullptr;
  // state
  zd *G = nullptr, *Gw = nullptr, *T1 = nullptr;
  zd *S = nullptr, *Sinv = nullptr;
  UDVSet udvl, udvr;
  std::vector<UDVSet> udvst;  // index nst-1
  // stabilisation work
  zd *TP = nullptr, *Qb = nullptr, *RHS = nullptr, *tau = nullptr, *Vtmp = nullptr, *dphase = nullptr;
  zd* QRw = nullptr;         // factored matrix (R above, reflectors below) of the last QR
  zd* gws = nullptr;         // split-K partial products of k_zgemm
  long long gws_elems = 0;
  double* qkeys = nullptr;   // column keys of the pre-pivoting
  int *jpvt = nullptr, *perm = nullptr, *iperm = nullptr;
  double *DUP = nullptr, *vn = nullptr, *cmp = nullptr, *opang = nullptr;
  QRInfo* info = nullptr;
  // delayed update
  int *m = nullptr, *sites = nullptr;
  zd *W = nullptr, *X = nullptr, *Y = nullptr, *dlt = nullptr;
  // per chain
  zd* phase = nullptr;
  long long* cnt = nullptr;
  double* stat = nullptr;
  int* err = nullptr;
  double* draws = nullptr;
  unsigned long long *rngkey = nullptr, *rngctr = nullptr;
  std::vector<unsigned long long> h_key, h_ctr;
  // recording
  int recording = 0, rec_stab = 0;
  int8_t* rec_acc = nullptr;
  int rec_nstm = 0;  // stabilisation points the recording buffers hold
  zd *rec_ratio = nullptr, *rec_G = nullptr, *rec_Gw = nullptr, *rec_phase = nullptr;
  FieldTables ft;
  std::vector<void*> allocs;
  // phase profiling (CUDA events on the library stream)
  int profiling = 0;
  long long launches = 0;  // kernel launches issued by this handle
  std::vector<cudaEvent_t> ev_pool;
  size_t ev_used = 0;
  std::vector<int> prof_cat;  // category of event pair i (events 2i, 2i+1)
  double prof_ms[ALFGPU_PROF_N] = {0};
  long long prof_n[ALFGPU_PROF_N] = {0};
};

static cudaEvent_t prof_event(alfgpu_s* h) {
  if (h->ev_used == h->ev_pool.size()) {
    cudaEvent_t e;
    cudaEventCreate(&e);
    h->ev_pool.push_back(e);
  }
  return h->ev_pool[h->ev_used++];
}
static void prof_begin(alfgpu_s* h, int cat) {
  if (!h->profiling) return;
  h->prof_cat.push_back(cat);
  cudaEventRecord(prof_event(h), h->st);
}
static void prof_end(alfgpu_s* h) {
  if (!h->profiling) return;
  cudaEventRecord(prof_event(h), h->st);
}
static void prof_collect(alfgpu_s* h) {
  if (h->prof_cat.empty()) return;
  cudaStreamSynchronize(h->st);
  for (size_t i = 0; i < h->prof_cat.size(); ++i) {
    float ms = 0.f;
    cudaEventElapsedTime(&ms, h->ev_pool[2 * i], h->ev_pool[2 * i + 1]);
    h->prof_ms[h->prof_cat[i]] += ms;
    h->prof_n[h->prof_cat[i]] += 1;
  }
  h->prof_cat.clear();
  h->ev_used = 0;
}

#define CK(x)                                   \
  do {                                          \
    cudaError_t e_ = (x);                       \
    if (e_ != cudaSuccess) {                    \
      h->last_cuda = e_;                        \
      h->last_line = __LINE__;                  \
      return ALFGPU_ERROR_CUDA;                 \
    }                                           \
  } while (0)
#define CKL()           \
  do {                  \
    h->launches++;      \
    CK(cudaGetLastError()); \
  } while (0)
#define RET(x)                \
  do {                        \
    int r_ = (x);             \
    if (r_) return r_;        \
  } while (0)

// A kernel's dynamic shared-memory limit is one setting per process and device, shared by
// every handle: it is only ever raised, so a handle created later with smaller needs does
// not invalidate the launches of an earlier one.
template <typename K>
static cudaError_t raise_smem_limit(K* kernel, size_t bytes) {
  static std::mutex mu;
  static std::map<std::pair<const void*, int>, size_t> done;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  std::lock_guard<std::mutex> lock(mu);
  size_t& cur = done[std::make_pair((const void*)kernel, dev)];
  if (bytes <= cur) return cudaSuccess;
  e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
  if (e == cudaSuccess) cur = bytes;
  return e;
}

template <typename T>
static int dalloc(alfgpu_s* h, T** p, size_t count) {
  void* q = nullptr;
  CK(cudaMalloc(&q, count * sizeof(T) + 16));
  h->allocs.push_back(q);  // freed by alfgpu_destroy even if the clear below fails
  CK(cudaMemset(q, 0, count * sizeof(T) + 16));
  *p = (T*)q;
  return 0;
}

static void fill_tables(FieldTables& ft) {
  const double sq6 = 2.449489742783178098197284074705891391965947480656670128432692567;
  for (int s = -2; s <= 2; ++s) { ft.phi[0][s + 2] = (double)s; ft.gama[0][s + 2] = 1.0; }
  const double a = sqrt(2.0 * (3.0 + sq6)), bq = sqrt(2.0 * (3.0 - sq6));
  ft.phi[1][0] = -a; ft.phi[1][1] = -bq; ft.phi[1][2] = 0.0; ft.phi[1][3] = bq; ft.phi[1][4] = a;
  ft.gama[1][0] = 1.0 - sq6 / 3.0; ft.gama[1][1] = 1.0 + sq6 / 3.0; ft.gama[1][2] = 1.0;
  ft.gama[1][3] = 1.0 + sq6 / 3.0; ft.gama[1][4] = 1.0 - sq6 / 3.0;
  const int8_t fl[5][3] = {{-1, 1, 2}, {1, 2, -2}, {0, 0, 0}, {2, -2, -1}, {-2, -1, 1}};
  memcpy(ft.flip, fl, sizeof(fl));
  for (int t = 0; t < 2; ++t)
    for (int so = 0; so < 5; ++so)
      for (int sn = 0; sn < 5; ++sn) ft.grat[t][so][sn] = ft.gama[t][sn] / ft.gama[t][so];
}

static int cluster_size(int N) {
  if (N >= 256) return 16;
  if (N >= 128) return 8;
  if (N >= 64) return 4;
  if (N >= 32) return 2;
  return 1;
}

// Resident clusters of CL CTAs for k_qrp_rows on an N x N matrix (0: it does not fit), rows in
// shared memory or (grows) in the global workspace.  The shared-memory limits it raises are
// process-global and only ever raised.
static int qrr_clusters(int N, int CL, bool grows = false) {
  const size_t sm = qrr_smem_bytes(N, CL, grows);
  if (sm > 227 * 1024) return 0;
  if (grows) {
    if (raise_smem_limit(k_qrp_rows<ArD, true>, sm) != cudaSuccess ||
        (CL > 8 && cudaFuncSetAttribute(k_qrp_rows<ArD, true>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) !=
                       cudaSuccess)) {
      cudaGetLastError();
      return 0;
    }
  } else if (raise_smem_limit(k_qrp_rows<ArD>, sm) != cudaSuccess ||
             raise_smem_limit(k_qrp_rows<ArF>, sm) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  if (!grows && CL > 8 &&
      (cudaFuncSetAttribute(k_qrp_rows<ArD>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) != cudaSuccess ||
       cudaFuncSetAttribute(k_qrp_rows<ArF>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) != cudaSuccess)) {
    cudaGetLastError();
    return 0;
  }
  cudaLaunchConfig_t cfg;
  memset(&cfg, 0, sizeof(cfg));
  cfg.gridDim = dim3(CL, 1, 1);
  cfg.blockDim = dim3(256, 1, 1);
  cfg.dynamicSmemBytes = sm;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = CL; at[0].val.clusterDim.y = 1; at[0].val.clusterDim.z = 1;
  cfg.attrs = at; cfg.numAttrs = 1;
  int n = 0;
  if (cudaOccupancyMaxActiveClusters(&n, grows ? k_qrp_rows<ArD, true> : k_qrp_rows<ArD>, &cfg) != cudaSuccess) n = 0;
  cudaGetLastError();
  return n;
}

// Cluster size and row storage of the exact pivoted QR of B matrices N x N.  For each row
// storage, rows in shared memory (mode 1) and rows in a global workspace (mode 2), the cluster
// size is CL, or CL / 2 when full-size clusters would put more than two CTAs on every SM (the
// flags force either); the plan takes shared-memory rows unless the global-row layout needs
// fewer waves of clusters (its CTAs need little shared memory, so several share an SM), or
// ALFGPU_FLAG_QR_GLOBAL_ROWS asks for it.  Mode 0: neither fits.
static int qrr_plan(int N, int CL, int B, int flags, int dev, int* CLout) {
  int nsm = 152;
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  cudaGetLastError();
  int best = 0, best_cl = CL;
  long long best_waves = 0;
  for (int mode = (flags & ALFGPU_FLAG_QR_GLOBAL_ROWS) ? 2 : 1; mode <= 2; ++mode) {
    const bool grows = mode == 2;
    int cl = CL, active = qrr_clusters(N, CL, grows);
    if (active <= 0) continue;
    if (CL >= 4) {
      const bool want = (flags & ALFGPU_FLAG_QR_HALF_CLUSTER) ||
                        (!(flags & ALFGPU_FLAG_QR_FULL_CLUSTER) && (long long)B * CL > 2ll * nsm);
      const int a2 = want ? qrr_clusters(N, CL / 2, grows) : 0;
      if (a2 > 0) { cl = CL / 2; active = a2; }
    }
    const long long waves = (B + active - 1) / active;
    if (!best || waves < best_waves) { best = mode; best_cl = cl; best_waves = waves; }
  }
  *CLout = best_cl;
  return best;
}

// One launch of the exact pivoted QR on clusters of CL CTAs (rows in shared memory, or in ws when
// grows), then k_bqr_finish: R (normalised rows) above, reflectors below, tau, jpvt, D, info.
static int launch_qrr(alfgpu_s* h, const zd* Ain, zd* A, int N, int CL, bool grows, zd* ws, zd* tau, int* jpvt,
                      double* D, QRInfo* info, const double* colscale, int df) {
  const int B = h->B;
  const long long NN = (long long)N * N;
  QRRowsParams q;
  memset(&q, 0, sizeof(q));
  q.Ain = Ain; q.A = A; q.lda = N; q.sA = NN; q.N = N;
  q.Araw = df ? h->QRdf : nullptr;
  q.colscale = colscale; q.sCS = N;
  q.tau = tau; q.sT = N; q.jpvt = jpvt; q.sP = N; q.D = D; q.sD = N; q.info = info;
  q.Arows = grows ? ws : nullptr;
  q.two_pass = (h->d.reserved[0] & ALFGPU_FLAG_QR_TWO_PASS) ? 1 : 0;
  cudaLaunchConfig_t cfg;
  memset(&cfg, 0, sizeof(cfg));
  cfg.gridDim = dim3(CL, B, 1);
  cfg.blockDim = dim3(256, 1, 1);
  cfg.dynamicSmemBytes = qrr_smem_bytes(N, CL, grows);
  cfg.stream = h->st;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = CL; at[0].val.clusterDim.y = 1; at[0].val.clusterDim.z = 1;
  cfg.attrs = at; cfg.numAttrs = 1;
  h->launches++;
  if (grows) CK(cudaLaunchKernelEx(&cfg, k_qrp_rows<ArD, true>, q));
  else if (df) CK(cudaLaunchKernelEx(&cfg, k_qrp_rows<ArF>, q));
  else CK(cudaLaunchKernelEx(&cfg, k_qrp_rows<ArD>, q));
  k_bqr_finish<<<dim3((N + 7) / 8, B), 256, (size_t)N * sizeof(double), h->st>>>(A, N, NN, N, tau, N, D, N, info);
  CKL();
  return 0;
}

// ---------------------------------------------------------------------------
// Kernel launch helpers
// ---------------------------------------------------------------------------
static int launch_qr(alfgpu_s* h, zd* A, const double* colscale, int nb) {
  prof_begin(h, ALFGPU_PROF_QR);
  QRParams q;
  memset(&q, 0, sizeof(q));
  const int N = h->N;
  q.A = A; q.lda = N; q.sA = (long long)N * N; q.N = N;
  q.tau = h->tau; q.sT = N;
  q.jpvt = h->jpvt; q.sP = N;
  q.D = h->DUP; q.sD = N;
  q.vn = h->vn; q.sV = 2 * N;
  q.colscale = colscale; q.sCS = N;
  q.info = h->info;
  cudaLaunchConfig_t cfg;
  memset(&cfg, 0, sizeof(cfg));
  cfg.gridDim = dim3(h->CL, nb, 1);
  cfg.blockDim = dim3(QR_THREADS, 1, 1);
  cfg.dynamicSmemBytes = (size_t)N * sizeof(zd);
  cfg.stream = h->st;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = h->CL; at[0].val.clusterDim.y = 1; at[0].val.clusterDim.z = 1;
  cfg.attrs = at; cfg.numAttrs = 1;
  h->launches++;
  CK(cudaLaunchKernelEx(&cfg, k_qrp, q));
  prof_end(h);
  return 0;
}

static int launch_orgqr(alfgpu_s* h, zd* A, int nb) {
  prof_begin(h, ALFGPU_PROF_ORGQR);
  OrgqrParams q;
  const int N = h->N;
  q.A = A; q.lda = N; q.sA = (long long)N * N; q.tau = h->tau; q.sT = N; q.N = N;
  cudaLaunchConfig_t cfg;
  memset(&cfg, 0, sizeof(cfg));
  cfg.gridDim = dim3(h->CL, nb, 1);
  cfg.blockDim = dim3(QR_THREADS, 1, 1);
  cfg.dynamicSmemBytes = (size_t)N * sizeof(zd);
  cfg.stream = h->st;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = h->CL; at[0].val.clusterDim.y = 1; at[0].val.clusterDim.z = 1;
  cfg.attrs = at; cfg.numAttrs = 1;
  h->launches++;
  CK(cudaLaunchKernelEx(&cfg, k_orgqr, q));
  prof_end(h);
  return 0;
}


// Triangular solves (ZTRSM) of p.nvec right-hand sides per matrix: TRSV_V vectors per CTA
// when their shared memory fits, else one per CTA.
static int trsv(alfgpu_s* h, const TrsvParams& t) {
  const size_t sm = trsv_v_smem(t.N);
  if (sm <= 200 * 1024 && raise_smem_limit(k_trsv_v<TRSV_V>, sm) == cudaSuccess) {
    k_trsv_v<TRSV_V><<<dim3((t.nvec + TRSV_V - 1) / TRSV_V, h->B), 256, sm, h->st>>>(t);
  } else {
    cudaGetLastError();
    k_trsv<<<dim3(t.nvec, h->B), 256, 3 * (size_t)t.N * sizeof(zd), h->st>>>(t);
  }
  return 0;  // the caller checks the launch (CKL)
}

static int gemm(alfgpu_s* h, const GemmParams& p) {
  int nl = 1;
  CK(launch_zgemm(p, h->st, h->gws, h->gws_elems, &nl));
  h->launches += nl;
  return 0;
}

static int gemm32(alfgpu_s* h, const GemmParams& g, int tA, int tB, int tC) {
  Gemm32Params P;
  P.g = g; P.tA = tA; P.tB = tB; P.tC = tC;
  h->launches++;
  CK(launch_dfgemm(P, h->st));
  return 0;
}

// Digit slices of one operand for k_oz_gemm (see ozaki.cuh for the modes).
static int oz_slice(alfgpu_s* h, const void* src, int mode, long long sr, long long sk, long long sb, int modb,
                    const zd* ks, long long sks, int srows, int Kc, const int* kdyn, int S, int bits, int Rpad,
                    int Kpad, unsigned short* out, int* expo, int batch) {
  OzSliceParams p;
  memset(&p, 0, sizeof(p));
  p.src = src; p.mode = mode; p.sr = sr; p.sk = sk; p.sb = sb; p.modb = modb;
  p.ks = ks; p.sks = sks; p.srows = srows; p.Kc = Kc; p.kdyn = kdyn;
  p.S = S; p.bits = bits; p.Rpad = Rpad; p.Kpad = Kpad; p.out = out; p.expo = expo; p.err = h->err;
  h->launches++;
  CK(oz_launch_slice(p, batch, h->st));
  return 0;
}

// C (M x Nn logical) = A B from two slice buffers; omode / osub as in OzGemmParams.
static int oz_gemm(alfgpu_s* h, const CUtensorMap& ta, const CUtensorMap& tb, int M, int Nn, int Kpad, int S,
                   int bits, int bn, int nst, int RpadA, int RpadB, int modA, int modB, const int* expA,
                   const int* expB, int omode, int osub, void* out, long long ldr, long long ldc, long long sout,
                   int batch, const zd* rsc = nullptr, long long srsc = 0, int SbA = 0, int SbB = 0,
                   const zd* csc = nullptr, long long scsc = 0, int persist_ctas = 0) {
  OzGemmParams p;
  memset(&p, 0, sizeof(p));
  p.M = M; p.N = Nn; p.nkc = Kpad / OZ_KC; p.S = S; p.bits = bits; p.nst = nst; p.nd = S + 1;
  p.SbA = SbA > 0 ? SbA : S; p.SbB = SbB > 0 ? SbB : S;
  p.csc = csc; p.scsc = scsc;
  p.L = oz_shift(Kpad, bits, S, p.nd);
  p.RpadA = RpadA; p.RpadB = RpadB; p.modA = modA; p.modB = modB; p.expA = expA; p.expB = expB;
  p.omode = omode; p.osub = osub; p.out = out; p.ldr = ldr; p.ldc = ldc; p.sout = sout; p.err = h->err;
  p.rsc = rsc; p.srsc = srsc;
  dim3 grid((Nn + bn - 1) / bn, (M + OZ_BM - 1) / OZ_BM, batch);
  const long long ntile = (long long)grid.x * grid.y * grid.z;
  if (persist_ctas > 0 && ntile > persist_ctas) {  // a bounded grid, each CTA looping over tiles
    p.persist = 1; p.tiles_n = (int)grid.x; p.tiles_m = (int)grid.y; p.tiles_b = (int)grid.z;
    grid = dim3((unsigned)persist_ctas, 1, 1);
  }
  const size_t sm = oz_smem_bytes(bn, S, p.nkc, nst);
  if (p.persist) {
    if (bn == 32) k_oz_gemm<32, true><<<grid, 256, sm, h->st>>>(ta, tb, p);
    else k_oz_gemm<16, true><<<grid, 256, sm, h->st>>>(ta, tb, p);
  } else if (bn == 32) {
    k_oz_gemm<32><<<grid, 256, sm, h->st>>>(ta, tb, p);
  } else {
    k_oz_gemm<16><<<grid, 256, sm, h->st>>>(ta, tb, p);
  }
  h->launches++;
  CKL();
  return 0;
}

// Slices of expT / expTinv (real, per flavour) as the M-side (rows i, K = columns) and
// N-side operand (rows j = output columns, K = rows).
static int oz_slice_expT(alfgpu_s* h) {
  if (!h->oz) return 0;
  const int N = h->N;
  const long long NN = (long long)N * N;
  const double* src[2] = {h->expT, h->expTinv};
  for (int a = 0; a < 2; ++a) {
    RET(oz_slice(h, src[a], OZ_REAL, 1, N, NN, 0, nullptr, 0, N, N, nullptr, h->oz_S, h->oz_bits, h->oz_RpN,
                 h->oz_Kpad, h->ozE[a], h->ozEe[a], h->F));
    RET(oz_slice(h, src[a], OZ_REAL, N, 1, NN, 0, nullptr, 0, N, N, nullptr, h->oz_S, h->oz_bits, h->oz_RpN,
                 h->oz_Kpad, h->ozE[2 + a], h->ozEe[2 + a], h->F));
  }
  return 0;
}

// Complex products of the stabilisation (CGR's U_R^H U_L, D_R V_R V_L D_L + RHS, the Q / U
// products with 1/DUP scales and pivot permutations; decompose's R P V) on the tensor-core
// GEMM in the mixed form: both operands as interleaved real / imaginary rows, the output
// row / column scales folded into the digit exponents of A's rows / B's rows, the four real
// products combined in the epilogue.  The real parts of rs / cs are used (the call sites pass
// real singular values); alpha = 1, beta in {0, 1}, square N x N x N only.
static bool oz_stab_ok(alfgpu_s* h, const GemmParams& g) {
  return h->mixed && h->oz && h->oz_stab && !g.realA && !g.realB && !g.ks && !g.kdyn && g.modA == 0 &&
         g.modB == 0 && g.alpha.x == 1.0 && g.alpha.y == 0.0 && g.beta.y == 0.0 &&
         (g.beta.x == 0.0 || g.beta.x == 1.0) && g.m == h->N && g.n == h->N && g.k == h->N && g.opA != OP_T &&
         g.opB != OP_T && g.batch == h->B;
}

static int oz_zgemm(alfgpu_s* h, const GemmParams& g) {
  const int N = h->N;
  OzSliceParams a;
  memset(&a, 0, sizeof(a));
  a.src = g.A; a.mode = OZ_CROWS; a.sb = g.sA; a.srows = N; a.Kc = N;
  if (g.opA == OP_N) { a.sr = 1; a.sk = g.lda; a.trans = 0; }
  else { a.sr = g.lda; a.sk = 1; a.trans = 1; a.conj = 1; }  // op(A)(i, k) = conj(A(k, i))
  a.perm = g.permA; a.sperm = g.sPA; a.tri = g.triA;
  a.rsc = g.rs; a.srsc = g.sRS; a.rinv = g.rsInv;
  a.S = h->oz_S; a.bits = h->oz_bits; a.Rpad = h->oz_Rp2N; a.Kpad = h->oz_Kpad;
  a.out = h->ozGA; a.expo = h->ozGAe; a.err = h->err;
  OzSliceParams bq = a;
  bq.src = g.B; bq.sb = g.sB;
  if (g.opB == OP_N) { bq.sr = g.ldb; bq.sk = 1; bq.trans = 1; bq.conj = 0; }  // op(B)(k, j) = B(k, j)
  else { bq.sr = 1; bq.sk = g.ldb; bq.trans = 0; bq.conj = 1; }              // op(B)(k, j) = conj(B(j, k))
  bq.perm = g.permB; bq.sperm = g.sPB; bq.tri = g.triB;
  bq.rsc = g.cs; bq.srsc = g.sCS; bq.rinv = g.csInv;
  bq.out = h->ozGB; bq.expo = h->ozGBe;
  h->launches += 2;
  CK(oz_launch_slice(a, h->B, h->st));
  CK(oz_launch_slice(bq, h->B, h->st));
  return oz_gemm(h, h->tmGA, h->tmGB, 2 * N, 2 * N, h->oz_Kpad, h->oz_S, h->oz_bits, h->oz_bn, h->oz_nst,
                 h->oz_Rp2N, h->oz_Rp2N, 0, 0, h->ozGAe, h->ozGBe, OZ_OUT_CPLX, g.beta.x == 1.0 ? -1 : 0, g.C, 1,
                 g.ldc, g.sC, h->B);
}

// The mixed form's UDV propagation runs on the tensor-core GEMM (FP64-accurate) when the
// slice scales are real.
static bool oz_propagate(alfgpu_s* h) {
  return h->mixed && h->oz && (!h->eexp_complex || h->pairblock) && !h->mixed_propagate;
}

// Stabilisation products (UDV propagation, decompose, CGR): double-float in the mixed
// form, FP64 otherwise.
static int gemm_s(alfgpu_s* h, const GemmParams& g) {
  if (oz_stab_ok(h, g)) return oz_zgemm(h, g);
  if (!h->df_stab) return gemm(h, g);
  return gemm32(h, g, g.realA ? ST_R64 : ST_C128, g.realB ? ST_R64 : ST_C128, ST_C128);
}

static GemmParams gsq(alfgpu_s* h, int batch) {  // N x N x N square product, batch strides N*N
  GemmParams p = gemm_defaults();
  const int N = h->N;
  p.m = p.n = p.k = N;
  p.lda = p.ldb = p.ldc = N;
  p.sA = p.sB = p.sC = (long long)N * N;
  p.batch = batch;
  return p;
}

static void drop_graphs(alfgpu_s* h) {
  for (int g = 0; g < 2; ++g)
    if (h->gexec[g]) { cudaGraphExecDestroy(h->gexec[g]); h->gexec[g] = nullptr; }
}

static int copy_mats(alfgpu_s* h, zd* dst, const zd* src, size_t count) {
  CK(cudaMemcpyAsync(dst, src, count * sizeof(zd), cudaMemcpyDeviceToDevice, h->st));
  return 0;
}

// count matrices X <- W X W^T (rotated basis -> original basis); no-op without two-site vertices
static int rotate_out(alfgpu_s* h, zd* X, int count) {
  if (!h->rot || count <= 0) return 0;
  const int np = (int)h->rot_pairs.size();
  dim3 grid((unsigned)(((long long)h->N * np + 255) / 256), count);
  const double* U = h->rot_U;
  k_rot_rows<<<grid, 256, 0, h->st>>>(X, h->N, h->rot_dev, np, U[0], U[1], U[2], U[3]);
  CKL();
  k_rot_cols<<<grid, 256, 0, h->st>>>(X, h->N, h->rot_dev, np, U[0], U[1], U[2], U[3]);
  CKL();
  return 0;
}

static int udv_copy(alfgpu_s* h, UDVSet& dst, const UDVSet& src) {
  const size_t NN = (size_t)h->N * h->N, B = h->B;
  RET(copy_mats(h, dst.U, src.U, B * NN));
  RET(copy_mats(h, dst.V, src.V, B * NN));
  CK(cudaMemcpyAsync(dst.D, src.D, B * h->N * sizeof(double), cudaMemcpyDeviceToDevice, h->st));
  CK(cudaMemcpyAsync(dst.detU, src.detU, B * sizeof(zd), cudaMemcpyDeviceToDevice, h->st));
  return 0;
}

static int udv_reset(alfgpu_s* h, UDVSet& s) {
  const int N = h->N;
  dim3 grid((unsigned)(((long long)N * N + 255) / 256), h->B);
  k_udv_reset<<<grid, 256, 0, h->st>>>(s.U, s.V, s.D, s.detU, N);
  CKL();
  return 0;
}

// Slice scale vectors S / Sinv of slice nt1 from the current fields.
static int slice_scale(alfgpu_s* h, int nt1) {
  k_slice_scale<<<h->B, 256, 0, h->st>>>(h->fields, h->L, h->M, h->N, h->F, nt1, h->v_sptr, h->v_slist, h->v_Eexp,
                                         h->S, h->Sinv);
  CKL();
  return 0;
}

// decompose_UDV_state (udv_state_mod.F90:466-578) on all B pairs; s.U holds the propagated A.
// QR of Ain * diag(colscale) into Aout (Aout != Ain): R above the diagonal (rows
// normalised by D = DUP), reflectors below, tau, jpvt, info.
static int wy_apply(alfgpu_s* h, const zd* F, int j0, int w, zd* C, int ncol, int adj);

static int qr_any(alfgpu_s* h, const zd* Ain, const double* colscale, zd* Aout, int exact, int df = 0) {
  const int N = h->N, B = h->B;
  const long long NN = (long long)N * N;
  h->exact_qrp = exact;
  h->qr_df = 0;
  const dim3 g8((N + 7) / 8, B);
  if (exact && !h->qrr_ok) {
    RET(copy_mats(h, Aout, Ain, (size_t)B * NN));
    return launch_qr(h, Aout, colscale, B);
  }
  prof_begin(h, ALFGPU_PROF_QR);
  if (exact) {
    const bool grows = h->qrr_ok == 2;
    RET(launch_qrr(h, Ain, Aout, N, h->CLr, grows, h->qrr_ws, h->tau, h->jpvt, h->DUP, h->info, colscale,
                   grows ? 0 : df));
    h->qr_df = grows ? 0 : df;
    prof_end(h);
    return 0;
  }
  k_bqr_keys<<<g8, 256, 0, h->st>>>(Ain, N, NN, N, colscale, N, h->qkeys);
  CKL();
  k_bqr_permute<<<g8, 256, (size_t)N * (sizeof(double) + sizeof(int)), h->st>>>(Ain, N, NN, N, colscale, N, h->qkeys,
                                                                                  Aout, NN, h->jpvt, N, h->info);
  CKL();
  for (int j0 = 0; j0 < N; j0 += BQR_NB) {
    const int w = (N - j0 < BQR_NB) ? N - j0 : BQR_NB;
    BQRPanel pp;
    pp.A = Aout; pp.lda = N; pp.sA = NN; pp.N = N; pp.j0 = j0; pp.nb = w;
    pp.tau = h->tau; pp.sT = N; pp.D = h->DUP; pp.sD = N;
    cudaLaunchConfig_t cfg;
    memset(&cfg, 0, sizeof(cfg));
    cfg.gridDim = dim3(h->CL, B, 1);
    cfg.blockDim = dim3(256, 1, 1);
    cfg.stream = h->st;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = h->CL; at[0].val.clusterDim.y = 1; at[0].val.clusterDim.z = 1;
    cfg.attrs = at; cfg.numAttrs = 1;
    h->launches++;
    CK(cudaLaunchKernelEx(&cfg, k_bqr_panel, pp));
    if (j0 + w < N) {
      BQRApply ap;
      ap.V = Aout; ap.ldv = N; ap.sV = NN; ap.tau = h->tau; ap.sT = N;
      ap.C = Aout; ap.ldc = N; ap.sC = NN;
      ap.N = N; ap.j0 = j0; ap.nb = w; ap.c0 = j0 + w; ap.conj_tau = 1; ap.init = 0;
      bqr_apply<ArD>(ap, dim3(N - j0 - w, B), h->st);
      CKL();
    }
  }
  k_bqr_finish<<<g8, 256, (size_t)N * sizeof(double), h->st>>>(Aout, N, NN, N, h->tau, N, h->DUP, N, h->info);
  CKL();
  h->qr_df = 0;
  prof_end(h);
  return 0;
}

// Explicit Q (first N columns of H_1 ... H_N) of the factored matrix F into Q (Q != F).
// One panel of w <= 32 Householder reflectors (columns j0 .. j0+w-1 of F: unit lower
// trapezoid V, tau) applied in compact-WY form to the ncol columns starting at C (ld N):
// C <- (I - V T V^H) C (adj = 0, ZUNGQR's H_j0 ... H_{j0+w-1}) or (I - V T^H V^H) C
// (adj = 1, the QR trailing update with H^H).  The Gram matrix V^H V and W = V^H C are
// digit-sliced tensor-core products, T follows ZLARFT's forward columnwise recursion,
// X = V T (or V T^H) is formed directly, and C -= X W is the flush's digit-sliced rank-w
// product.
static int wy_apply(alfgpu_s* h, const zd* F, int j0, int w, zd* C, int ncol, int adj) {
  const int N = h->N, B = h->B;
  const long long NN = (long long)N * N;
  const int S = h->oz_S, bits = h->oz_bits, Kp = h->oz_Kpad, Rp2 = h->oz_Rp2N, bn = h->oz_bn, nst = h->oz_nst;
  OzSliceParams a;
  memset(&a, 0, sizeof(a));
  a.src = F + (long long)j0 * N; a.mode = OZ_CROWS; a.sb = NN; a.srows = w; a.Kc = N;
  a.sr = N; a.sk = 1; a.trans = 1; a.conj = 1; a.unitlow = 1; a.doff = j0;  // op C of V
  a.S = S; a.bits = bits; a.Rpad = Rp2; a.Kpad = Kp; a.out = h->ozGA; a.expo = h->ozGAe; a.err = h->err;
  OzSliceParams v = a;
  v.conj = 0; v.out = h->ozGB; v.expo = h->ozGBe;  // V itself as the N-side operand
  h->launches += 2;
  CK(oz_launch_slice(a, B, h->st));
  CK(oz_launch_slice(v, B, h->st));
  RET(oz_gemm(h, h->tmGA, h->tmGB, 2 * w, 2 * w, Kp, S, bits, bn, nst, Rp2, Rp2, 0, 0, h->ozGAe, h->ozGBe,
              OZ_OUT_CPLX, 0, h->ozGm, 1, 32, 1024, B));
  k_bqr_larft<<<B, 256, 0, h->st>>>(h->ozGm, h->tau, N, j0, w, h->ozTm);
  CKL();
  OzSliceParams cs = a;  // C as the N-side operand: row j = column j of C, K = rows
  cs.src = C; cs.srows = ncol; cs.conj = 0; cs.unitlow = 0; cs.out = h->ozGB; cs.expo = h->ozGBe;
  h->launches++;
  CK(oz_launch_slice(cs, B, h->st));
  RET(oz_gemm(h, h->tmGA, h->tmGB, 2 * w, 2 * ncol, Kp, S, bits, bn, nst, Rp2, Rp2, 0, 0, h->ozGAe, h->ozGBe,
              OZ_OUT_CPLX, 0, h->ozWm, 1, 32, 32ll * N, B));
  k_bqr_vt<<<dim3((N + 7) / 8, B), dim3(32, 8), 0, h->st>>>(F, N, NN, h->ozTm, N, j0, w, h->ozXm, 32ll * N, adj);
  CKL();
  // C -= X W: [Re X | Im X] times the K-doubled rows of W (the flush's product)
  OzSliceParams xa;
  memset(&xa, 0, sizeof(xa));
  xa.src = h->ozXm; xa.mode = OZ_CKA; xa.sr = 1; xa.sk = N; xa.sb = 32ll * N; xa.srows = N; xa.Kc = 32;
  xa.kvalid = w; xa.S = h->ozf_S; xa.bits = h->ozf_bits; xa.Rpad = h->oz_RpN; xa.Kpad = 64; xa.out = h->ozXA;
  xa.expo = h->ozXAe; xa.err = h->err;
  OzSliceParams yb = xa;
  yb.src = h->ozWm; yb.mode = OZ_CKB; yb.sr = 32; yb.sk = 1; yb.srows = ncol; yb.Rpad = Rp2; yb.out = h->ozYB;
  yb.expo = h->ozYBe;
  h->launches += 2;
  CK(oz_launch_slice(xa, B, h->st));
  CK(oz_launch_slice(yb, B, h->st));
  return oz_gemm(h, h->tmXA, h->tmYB, N, 2 * ncol, 64, h->ozf_S, h->ozf_bits, h->ozf_bn, h->ozf_nst, h->oz_RpN, Rp2,
                 0, 0, h->ozXAe, h->ozYBe, OZ_OUT_COLS, 1, C, 1, N, NN, B, nullptr, 0, 0, 0, nullptr, 0, h->ozf_grid);
}

// Explicit Q (ZUNGQR) in compact-WY form on the tensor-core GEMM (mixed form, batched
// grids): Q starts as the identity and the panels are applied from the last to the first
// to the columns from their first one on (the columns of a panel are still e_c then).
static int orgqr_wy(alfgpu_s* h, const zd* F, zd* Q) {
  const int N = h->N, B = h->B;
  const long long NN = (long long)N * N;
  prof_begin(h, ALFGPU_PROF_ORGQR);
  k_bqr_eye<<<dim3((unsigned)((NN + 255) / 256), B), 256, 0, h->st>>>(Q, N, NN);
  CKL();
  for (int j0 = ((N - 1) / 32) * 32; j0 >= 0; j0 -= 32) {
    const int w = (N - j0 < 32) ? N - j0 : 32;
    RET(wy_apply(h, F, j0, w, Q + (long long)j0 * N, N - j0, 0));
  }
  prof_end(h);
  return 0;
}

static int orgqr_any(alfgpu_s* h, const zd* F, zd* Q) {
  const int N = h->N, B = h->B;
  const long long NN = (long long)N * N;
  // compact WY pays on batched grids; one chain's grid is too small for its launch chain
  if (h->oz_stab && !h->oz_narrow && !h->qr_df && N <= 32 * BQR_LROWS) return orgqr_wy(h, F, Q);
  if (N > 32 * BQR_LROWS) {  // beyond the rows a lane of k_bqr_apply holds
    RET(copy_mats(h, Q, F, (size_t)B * NN));
    return launch_orgqr(h, Q, B);
  }
  prof_begin(h, ALFGPU_PROF_ORGQR);
  for (int j0 = ((N - 1) / BQR_NB) * BQR_NB; j0 >= 0; j0 -= BQR_NB) {
    const int w = (N - j0 < BQR_NB) ? N - j0 : BQR_NB;
    BQRApply ap;
    ap.V = h->qr_df ? (const void*)h->QRdf : (const void*)F; ap.ldv = N; ap.sV = NN; ap.tau = h->tau; ap.sT = N;
    ap.C = Q; ap.ldc = N; ap.sC = NN;
    ap.N = N; ap.j0 = j0; ap.nb = w; ap.c0 = j0; ap.conj_tau = 0; ap.init = 1;
    if (h->qr_df) bqr_apply<ArF>(ap, dim3(N - j0, B), h->st);
    else bqr_apply<ArD>(ap, dim3(N - j0, B), h->st);
    CKL();
  }
  prof_end(h);
  return 0;
}

// Decompose with ZGEQP3 in place on s.U (no work matrix): the allocation-free entry point.
static int decompose_inplace(alfgpu_s* h, UDVSet& s, int left) {
  const int N = h->N, B = h->B;
  const long long NN = (long long)N * N;
  RET(launch_qr(h, s.U, s.D, B));
  k_decomp_phase<<<B, 256, 0, h->st>>>(s.U, N, N, h->info, left, h->dphase, s.detU);
  CKL();
  k_perm0<<<dim3((N + 255) / 256, B), 256, 0, h->st>>>(h->jpvt, N, h->perm, N, N);
  CKL();
  GemmParams p = gsq(h, B);
  if (!left) {  // V = R * P^T V   (ZLAPMR forward, ZTRMM L,U,N)
    p.A = s.U; p.opA = OP_N; p.triA = 1;
    p.B = s.V; p.opB = OP_N; p.permB = h->perm; p.sPB = N;
  } else {      // V = (V P) * R^H (ZLAPMT forward, ZTRMM R,U,C)
    p.A = s.V; p.opA = OP_N; p.permA = h->perm; p.sPA = N;
    p.B = s.U; p.opB = OP_C; p.triB = 1;
  }
  p.C = h->Vtmp;
  RET(gemm(h, p));
  RET(copy_mats(h, s.V, h->Vtmp, (size_t)B * NN));
  CK(cudaMemcpyAsync(s.D, h->DUP, (size_t)B * N * sizeof(double), cudaMemcpyDeviceToDevice, h->st));
  RET(launch_orgqr(h, s.U, B));
  k_scale_col0<<<B, 256, 0, h->st>>>(s.U, N, h->dphase);
  CKL();
  return 0;
}

// decompose_UDV_state (udv_state_mod.F90:448-582): QR of U*D, phase of det(R) moved into U(:,1),
// V <- R P^-1 V, U <- Q.  The factored matrix goes to the work matrix QRw; Q is formed into s.U.
static int decompose(alfgpu_s* h, UDVSet& s, int left) {
  if (!h->QRw) return decompose_inplace(h, s, left);
  const int N = h->N, B = h->B;
  RET(qr_any(h, s.U, s.D, h->QRw, h->exact_dec, h->df_qr && h->exact_dec));
  k_decomp_phase<<<B, 256, 0, h->st>>>(h->QRw, N, N, h->info, left, h->dphase, s.detU);
  CKL();
  k_perm0<<<dim3((N + 255) / 256, B), 256, 0, h->st>>>(h->jpvt, N, h->perm, N, N);
  CKL();
  GemmParams p = gsq(h, B);
  if (!left) {  // V = R * P^T V   (ZLAPMR forward, ZTRMM L,U,N)
    p.A = h->QRw; p.opA = OP_N; p.triA = 1;
    p.B = s.V; p.opB = OP_N; p.permB = h->perm; p.sPB = N;
  } else {      // V = (V P) * R^H (ZLAPMT forward, ZTRMM R,U,C)
    p.A = s.V; p.opA = OP_N; p.permA = h->perm; p.sPA = N;
    p.B = h->QRw; p.opB = OP_C; p.triB = 1;
  }
  p.C = h->Vtmp;
  RET(gemm_s(h, p));
  RET(copy_mats(h, s.V, h->Vtmp, (size_t)B * N * N));  // buffer roles stay fixed (graph replay)
  CK(cudaMemcpyAsync(s.D, h->DUP, (size_t)B * N * sizeof(double), cudaMemcpyDeviceToDevice, h->st));
  RET(orgqr_any(h, h->QRw, s.U));
  k_scale_col0<<<B, 256, 0, h->st>>>(s.U, N, h->dphase);
  CKL();
  return 0;
}

// Explicit wraps of vertex phase ph on the B matrices X: left (rows) or right (columns)
// multiplication by E_ph(s) (inv = 0) or E_ph(-s) (inv = 1), entries conjugated with cj; the
// fields of slice nt1, or the snapshot of the slice's fields before its updates (snap).
static int vtx_phase(alfgpu_s* h, zd* X, int ph, int nt1, bool snap, int inv, int cj, bool rows) {
  VtxPhase p;
  p.fl = snap ? h->fields_old : h->fields + (long long)(nt1 - 1) * h->M;
  p.fstride = snap ? h->M : (long long)h->L * h->M;
  p.kind = h->v_kind; p.site = h->v_site; p.site2 = h->v_blk2; p.coef = h->v_vc; p.Eexp = h->v_Eexp;
  p.sK = (long long)h->F * h->M; p.F = h->F; p.M = h->M; p.N = h->N;
  p.n0 = h->ph_n0[ph]; p.n1 = h->ph_n1[ph]; p.inv = inv; p.cj = cj;
  const long long nthr = (long long)h->N * (p.n1 - p.n0);
  const dim3 grid((unsigned)((nthr + 255) / 256), h->B);
  const long long NN = (long long)h->N * h->N;
  if (rows) k_vtx_rows<<<grid, 256, 0, h->st>>>(X, NN, p);
  else k_vtx_cols<<<grid, 256, 0, h->st>>>(X, NN, p);
  CKL();
  return 0;
}
// The slice's vertex product P = E_K ... E_1 (phases in visit order, fields of slice nt1):
// X <- P X, X <- P^dagger X, X <- X P^-1.
static int vtx_left(alfgpu_s* h, zd* X, int nt1) {
  for (size_t ph = 0; ph < h->ph_n0.size(); ++ph) RET(vtx_phase(h, X, (int)ph, nt1, false, 0, 0, true));
  return 0;
}
static int vtx_left_adj(alfgpu_s* h, zd* X, int nt1) {
  for (int ph = (int)h->ph_n0.size() - 1; ph >= 0; --ph) RET(vtx_phase(h, X, ph, nt1, false, 0, 1, true));
  return 0;
}
static int vtx_right_inv(alfgpu_s* h, zd* X, int nt1) {
  for (size_t ph = 0; ph < h->ph_n0.size(); ++ph) RET(vtx_phase(h, X, (int)ph, nt1, false, 1, 0, false));
  return 0;
}

// Checkerboard hopping on the B matrices X (Hop_mod.F90:143-250 with the bond operators in Op_T
// order): each family's disjoint bonds in one launch, families in the order of the routine.
enum { CB_MMTHR, CB_MMTHR_M1, CB_MMTHL, CB_MMTHL_M1, CB_MMTHLC };
static int cb_apply(alfgpu_s* h, zd* X, int which) {
  const int nfam = (int)h->cb_fam.size() - 1;
  const bool rows = which == CB_MMTHR || which == CB_MMTHR_M1 || which == CB_MMTHLC;
  const bool inv = which == CB_MMTHR_M1 || which == CB_MMTHL_M1;
  const bool reverse = which == CB_MMTHR || which == CB_MMTHL_M1;  // the last family first
  const long long NN = (long long)h->N * h->N;
  for (int q = 0; q < nfam; ++q) {
    const int fm = reverse ? nfam - 1 - q : q;
    const int b0 = h->cb_fam[fm], b1 = h->cb_fam[fm + 1];
    if (b1 <= b0) continue;
    const dim3 grid((unsigned)(((long long)h->N * (b1 - b0) + 255) / 256), h->B);
    if (rows)
      k_bond_rows<<<grid, 256, 0, h->st>>>(X, NN, h->N, h->F, h->cb_P, inv ? h->cb_inv : h->cb_mat, h->cb_ncheck, b0,
                                           b1);
    else
      k_bond_cols<<<grid, 256, 0, h->st>>>(X, NN, h->N, h->F, h->cb_P, inv ? h->cb_inv : h->cb_mat, h->cb_ncheck, b0,
                                           b1);
    CKL();
  }
  return 0;
}
static int scale_rc(alfgpu_s* h, zd* X, const zd* rs, int rconj, const zd* cs) {
  const dim3 grid((unsigned)(((long long)h->N * h->N + 255) / 256), h->B);
  k_scale_rc<<<grid, 256, 0, h->st>>>(X, h->N, rs, rconj, cs);
  CKL();
  return 0;
}

// WRAPUR (wrapur_mod.F90:101-124): U <- prod_nt [D_nt expT] U, then decompose (side R)
static int wrapur_u(alfgpu_s* h, UDVSet& u, int ntau, int ntau1) {
  const int N = h->N, B = h->B;
  prof_begin(h, ALFGPU_PROF_PROPAGATE);
  for (int nt = ntau + 1; nt <= ntau1; ++nt) {
    if (h->cb) {  // U <- P (B_T U) with the bond operators (Hop_mod_mmthr), then the vertices
      RET(cb_apply(h, u.U, CB_MMTHR));
      if (h->pairblock) {
        RET(vtx_left(h, u.U, nt));
      } else {
        RET(slice_scale(h, nt));
        RET(scale_rc(h, u.U, h->S, 0, nullptr));
      }
      continue;
    }
    if (h->pairblock) {  // U <- P (expT U): the product, then the slice's explicit vertex phases
      if (oz_propagate(h)) {
        RET(oz_slice(h, u.U, OZ_CROWS, N, 1, (long long)N * N, 0, nullptr, 0, N, N, nullptr, h->ozp_S, h->oz_bits,
                     h->oz_Rp2N, h->oz_Kpad, h->ozGB, h->ozGBe, B));
        RET(oz_gemm(h, h->tmE[0], h->tmGB, N, 2 * N, h->oz_Kpad, h->ozp_S, h->oz_bits, h->oz_bn, h->oz_nst,
                    h->oz_RpN, h->oz_Rp2N, h->F, 0, h->ozEe[0], h->ozGBe, OZ_OUT_COLS, 0, u.U, 1, N,
                    (long long)N * N, B, nullptr, 0, h->oz_S, h->ozp_S));
      } else {
        GemmParams p = gsq(h, B);
        p.A = h->expT; p.realA = 1; p.modA = h->F;
        p.B = u.U; p.C = h->T1;
        RET(gemm_s(h, p));
        RET(copy_mats(h, u.U, h->T1, (size_t)B * N * N));
      }
      RET(vtx_left(h, u.U, nt));
      continue;
    }
    RET(slice_scale(h, nt));
    if (oz_propagate(h)) {  // U <- diag(S) expT U on the tensor cores, in place (U is sliced first)
      RET(oz_slice(h, u.U, OZ_CROWS, N, 1, (long long)N * N, 0, nullptr, 0, N, N, nullptr, h->ozp_S, h->oz_bits,
                   h->oz_Rp2N, h->oz_Kpad, h->ozGB, h->ozGBe, B));
      RET(oz_gemm(h, h->tmE[0], h->tmGB, N, 2 * N, h->oz_Kpad, h->ozp_S, h->oz_bits, h->oz_bn, h->oz_nst, h->oz_RpN,
                  h->oz_Rp2N, h->F, 0, h->ozEe[0], h->ozGBe, OZ_OUT_COLS, 0, u.U, 1, N, (long long)N * N, B, h->S,
                  N, h->oz_S, h->ozp_S));
      continue;
    }
    GemmParams p = gsq(h, B);
    p.A = h->expT; p.realA = 1; p.modA = h->F;
    p.B = u.U; p.C = h->T1;
    p.rs = h->S; p.sRS = N;
    if (h->mixed_propagate) RET(gemm32(h, p, ST_R64, ST_C128, ST_C128));
    else RET(gemm_s(h, p));
    RET(copy_mats(h, u.U, h->T1, (size_t)B * N * N));
  }
  prof_end(h);
  return decompose(h, u, 0);
}
static int wrapur(alfgpu_s* h, int ntau, int ntau1) { return wrapur_u(h, h->udvr, ntau, ntau1); }

// WRAPUL (wrapul_mod.F90:108-131): U <- prod_nt [expT conj(D_nt)] U (descending nt), decompose (side L)
static int wrapul(alfgpu_s* h, int ntau1, int ntau) {
  const int N = h->N, B = h->B;
  prof_begin(h, ALFGPU_PROF_PROPAGATE);
  for (int nt = ntau1; nt >= ntau + 1; --nt) {
    if (h->cb) {  // U <- B_T^T (P^dagger U): the vertices, then the bonds (Hop_mod_mmthlc)
      if (h->pairblock) {
        RET(vtx_left_adj(h, h->udvl.U, nt));
      } else {
        RET(slice_scale(h, nt));
        RET(scale_rc(h, h->udvl.U, h->S, 1, nullptr));
      }
      RET(cb_apply(h, h->udvl.U, CB_MMTHLC));
      continue;
    }
    if (h->pairblock) {  // U <- expT (P^dagger U): the slice's explicit vertex phases, then the product
      RET(vtx_left_adj(h, h->udvl.U, nt));
      if (oz_propagate(h)) {
        RET(oz_slice(h, h->udvl.U, OZ_CROWS, N, 1, (long long)N * N, 0, nullptr, 0, N, N, nullptr, h->ozp_S,
                     h->oz_bits, h->oz_Rp2N, h->oz_Kpad, h->ozGB, h->ozGBe, B));
        RET(oz_gemm(h, h->tmE[0], h->tmGB, N, 2 * N, h->oz_Kpad, h->ozp_S, h->oz_bits, h->oz_bn, h->oz_nst,
                    h->oz_RpN, h->oz_Rp2N, h->F, 0, h->ozEe[0], h->ozGBe, OZ_OUT_COLS, 0, h->udvl.U, 1, N,
                    (long long)N * N, B, nullptr, 0, h->oz_S, h->ozp_S));
      } else {
        GemmParams q = gsq(h, B);
        q.A = h->expT; q.realA = 1; q.modA = h->F;
        q.B = h->udvl.U; q.C = h->T1;
        RET(gemm_s(h, q));
        RET(copy_mats(h, h->udvl.U, h->T1, (size_t)B * N * N));
      }
      continue;
    }
    RET(slice_scale(h, nt));
    if (oz_propagate(h)) {  // U <- expT diag(conj S) U on the tensor cores (S real), in place
      RET(oz_slice(h, h->udvl.U, OZ_CROWS, N, 1, (long long)N * N, 0, h->S, N, N, N, nullptr, h->ozp_S, h->oz_bits,
                   h->oz_Rp2N, h->oz_Kpad, h->ozGB, h->ozGBe, B));
      RET(oz_gemm(h, h->tmE[0], h->tmGB, N, 2 * N, h->oz_Kpad, h->ozp_S, h->oz_bits, h->oz_bn, h->oz_nst, h->oz_RpN,
                  h->oz_Rp2N, h->F, 0, h->ozEe[0], h->ozGBe, OZ_OUT_COLS, 0, h->udvl.U, 1, N, (long long)N * N, B,
                  nullptr, 0, h->oz_S, h->ozp_S));
      continue;
    }
    GemmParams q = gsq(h, B);
    q.A = h->expT; q.realA = 1; q.modA = h->F;
    q.B = h->udvl.U; q.C = h->T1;
    q.ks = h->S; q.sKS = N; q.ksConj = 1;
    if (h->mixed_propagate) RET(gemm32(h, q, ST_R64, ST_C128, ST_C128));
    else RET(gemm_s(h, q));
    RET(copy_mats(h, h->udvl.U, h->T1, (size_t)B * N * N));
  }
  prof_end(h);
  return decompose(h, h->udvl, 1);
}

// CGR default branch (cgr1_mod.F90:174-447) for all pairs into G; phase pieces into info/dphase.
static int cgr(alfgpu_s* h, int nvar, const UDVSet& ur, const UDVSet& ul, zd* Gout) {
  const int N = h->N, B = h->B;
  const long long NN = (long long)N * N;
  // RHS = U_R^H U_L
  {
    GemmParams p = gsq(h, B);
    p.A = ur.U; p.opA = OP_C; p.B = ul.U; p.opB = OP_N; p.C = h->RHS;
    RET(gemm_s(h, p));
  }
  // TPUP = D_R (V_R V_L) D_L + RHS  (D's packed as complex scale vectors in S / Sinv)
  RET(copy_mats(h, h->TP, h->RHS, (size_t)B * NN));
  k_real_to_complex2<<<(unsigned)((B * N + 255) / 256), 256, 0, h->st>>>(ur.D, ul.D, h->S, h->Sinv, (long long)B * N);
  CKL();
  {
    GemmParams p = gsq(h, B);
    p.A = ur.V; p.B = ul.V; p.C = h->TP; p.beta = zmk(1.0, 0.0);
    p.rs = h->S; p.sRS = N;
    p.cs = h->Sinv; p.sCS = N;
    RET(gemm_s(h, p));
  }
  zd* QR = h->TP;
  if (nvar != 1) {
    dim3 grid((N + 31) / 32, (N + 31) / 32, B);
    k_transpose<<<grid, dim3(32, 8), 0, h->st>>>(h->TP, N, NN, h->Qb, N, NN, N, 1);
    CKL();
    QR = h->Qb;
  }
  RET(qr_any(h, QR, nullptr, h->QRw, h->exact_cgr));
  zd* Q = QR;  // the input is no longer needed
  RET(orgqr_any(h, h->QRw, Q));
  QR = h->QRw;
  k_invperm<<<dim3((N + 255) / 256, B), 256, 0, h->st>>>(h->jpvt, N, h->iperm, N, N);
  CKL();
  k_real_to_complex<<<(B * N + 255) / 256, 256, 0, h->st>>>(h->DUP, h->S, (long long)B * N);
  CKL();
  if (nvar == 1) {
    // RHS = Q^H U_R^H, rows divided by DUP
    GemmParams p = gsq(h, B);
    p.A = Q; p.opA = OP_C; p.B = ur.U; p.opB = OP_C; p.C = h->RHS;
    p.rs = h->S; p.sRS = N; p.rsInv = 1;
    RET(gemm_s(h, p));
    // R y = RHS (ZTRSM L,U,N), columns of RHS
    TrsvParams t{};
    t.T = QR; t.ldt = N; t.sT = NN; t.B = h->RHS; t.vstride = N; t.estride = 1; t.sB = NN;
    t.N = N; t.nvec = N; t.lower = 0; t.conj_io = 0;
    prof_begin(h, ALFGPU_PROF_SOLVE);
    RET(trsv(h, t));
    prof_end(h);
    CKL();
    // G = U_L * P RHS (ZLAPMR backward folded into the B load)
    GemmParams g = gsq(h, B);
    g.A = ul.U; g.B = h->RHS; g.permB = h->iperm; g.sPB = N; g.C = Gout;
    RET(gemm_s(h, g));
  } else {
    // RHS = U_L Q, columns divided by DUP
    GemmParams p = gsq(h, B);
    p.A = ul.U; p.B = Q; p.C = h->RHS;
    p.cs = h->S; p.sCS = N; p.csInv = 1;
    RET(gemm_s(h, p));
    // y R^H = RHS (ZTRSM R,U,C): rows of RHS, conjugated, upper solve
    TrsvParams t{};
    t.T = QR; t.ldt = N; t.sT = NN; t.B = h->RHS; t.vstride = 1; t.estride = N; t.sB = NN;
    t.N = N; t.nvec = N; t.lower = 0; t.conj_io = 1;
    prof_begin(h, ALFGPU_PROF_SOLVE);
    RET(trsv(h, t));
    prof_end(h);
    CKL();
    // G = (RHS P) U_R^H (ZLAPMT backward folded into the A load)
    GemmParams g = gsq(h, B);
    g.A = h->RHS; g.permA = h->iperm; g.sPA = N; g.B = ur.U; g.opB = OP_C; g.C = Gout;
    RET(gemm_s(h, g));
  }
  return 0;
}


// One stabilisation: Gw = G (TEST), CGR into G, compare, phases (main.F90:734-753).
static int stabilise(alfgpu_s* h, int nvar, int compare) {
  const int N = h->N, B = h->B;
  const long long NN = (long long)N * N;
  if (compare) RET(copy_mats(h, h->Gw, h->G, (size_t)B * NN));
  RET(cgr(h, nvar, h->udvr, h->udvl, h->G));
  if (compare) {
    const zd* gnew = h->G;
    if (h->rot) {  // Control_PrecisionG in the original basis
      RET(copy_mats(h, h->TP, h->G, (size_t)B * NN));
      RET(rotate_out(h, h->TP, B));
      RET(rotate_out(h, h->Gw, B));
      gnew = h->TP;
    }
    CK(cudaMemsetAsync(h->cmp, 0, 2 * (size_t)B * sizeof(double), h->st));
    k_compare<<<dim3(CMP_BLOCKS, B), 256, 0, h->st>>>(gnew, h->Gw, N, h->cmp, h->err);
    CKL();
  }
  k_opphase<<<B, 256, 0, h->st>>>(h->fields, h->L, h->M, h->F, h->v_g, h->v_alpha, h->v_type, h->ft, h->opang);
  CKL();
  StabFinishParams sp;
  sp.C = h->C; sp.F = h->F; sp.NSUN = h->NSUN; sp.nvar = nvar; sp.compare = compare; sp.init = !compare;
  sp.detUR = h->udvr.detU; sp.detUL = h->udvl.detU; sp.info = h->info; sp.opang = h->opang; sp.cmp = h->cmp;
  sp.phase = h->phase; sp.stat = h->stat; sp.err = h->err;
  sp.rec_phase = nullptr;
  if (h->recording && compare) {
    sp.rec_phase = h->rec_phase + (long long)h->rec_stab * h->C;
    RET(copy_mats(h, h->rec_G + (long long)h->rec_stab * B * NN, h->G, (size_t)B * NN));
    RET(copy_mats(h, h->rec_Gw + (long long)h->rec_stab * B * NN, h->Gw, (size_t)B * NN));
    RET(rotate_out(h, h->rec_G + (long long)h->rec_stab * B * NN, B));  // Gw is already rotated
    h->rec_stab++;
  }
  k_stab_finish<<<(h->C + 127) / 128, 128, 0, h->st>>>(sp);
  CKL();
  return 0;
}

// ---- measurements ---------------------------------------------------------------------------
static int ensure_obs_host(alfgpu_s* h) {
  const size_t NN = (size_t)h->N * h->N;
  if (!h->obs_host) CK(cudaMallocHost(&h->obs_host, (size_t)h->B * NN * sizeof(zd)));
  if (!h->phase_host) CK(cudaMallocHost(&h->phase_host, (size_t)h->C * sizeof(zd)));
  if (h->ltau && !h->tau_host) CK(cudaMallocHost(&h->tau_host, 4 * (size_t)h->B * NN * sizeof(zd)));
  return 0;
}

// ham%Obser(GR, PHASE, ntau1) for every chain (main.F90:757-772, 788-803).  With a pending
// vertex scaling (up pass), G in ALF's frame is S G Sinv, formed into the work matrix Gw.
static LattObsParams latt_params(alfgpu_s* h, int kind) {
  LattObsParams p;
  p.N = h->N; p.F = h->F; p.nsun = h->NSUN; p.ncell = h->lo_ncell; p.norb = h->lo_norb; p.nnames = h->lo_nnames;
  p.L1 = kind ? h->L + 1 : 1;
  p.site_of = h->lo_site; p.jof = h->lo_jof; p.phase = h->phase;
  p.acc = h->lo_acc[kind]; p.acc0 = h->lo_acc0[kind]; p.cnt = h->lo_cnt[kind];
  return p;
}

static int obs_eq(alfgpu_s* h, alfgpu_obs_cb cb, void* ctx, int ntau1, int pending) {
  if (!cb && !h->obs_scal && !h->obs_latt) return 0;
  const long long NN = (long long)h->N * h->N;
  const zd* src = h->G;
  if (pending || h->rot) {
    RET(copy_mats(h, h->Gw, h->G, (size_t)h->B * NN));
    if (pending) {
      dim3 grid((unsigned)((NN + 255) / 256), h->B);
      k_apply_scale<<<grid, 256, 0, h->st>>>(h->Gw, h->S, h->Sinv, h->N);
      CKL();
    }
    RET(rotate_out(h, h->Gw, h->B));
    src = h->Gw;
  }
  if (h->obs_scal) {
    k_obs_scal<<<h->C, 256, 0, h->st>>>(src, h->phase, h->obs_HT, h->obs_trH, h->obs_U, h->N, h->F, h->obs_nsun,
                                        h->obs_acc);
    CKL();
  }
  if (h->obs_latt) {
    const int nout = h->lo_ncell * h->lo_norb * h->lo_norb;
    k_obs_latt_eq<<<dim3((nout + 127) / 128, h->C), 128, 0, h->st>>>(src, latt_params(h, 0));
    CKL();
  }
  if (!cb) return 0;
  RET(ensure_obs_host(h));
  CK(cudaMemcpyAsync(h->obs_host, src, (size_t)h->B * NN * sizeof(zd), cudaMemcpyDeviceToHost, h->st));
  CK(cudaMemcpyAsync(h->phase_host, h->phase, (size_t)h->C * sizeof(zd), cudaMemcpyDeviceToHost, h->st));
  CK(cudaStreamSynchronize(h->st));
  for (int c = 0; c < h->C; ++c)
    cb(ctx, c, ntau1, 0, h->obs_host + (size_t)c * h->F * NN * 2, h->phase_host + 2 * c);
  return 0;
}

// ham%ObserT(NT, GT0, G0T, G00, GTT, PHASE) for every chain (tau_m_mod.F90:116, 168)
static int obs_tau(alfgpu_s* h, alfgpu_obs_cb cb, void* ctx, int nt) {
  if (!cb && !h->obs_latt) return 0;
  const long long NN = (long long)h->N * h->N;
  dim3 grid((unsigned)((NN + 255) / 256), h->B);
  k_gather_quartet<<<grid, 256, 0, h->st>>>(h->GT0, h->G0T, h->G00, h->GTT, h->Gq, h->N, h->F);
  CKL();
  RET(rotate_out(h, h->Gq, 4 * h->B));
  if (h->obs_latt) {
    const int nout = h->lo_ncell * h->lo_norb * h->lo_norb;
    k_obs_latt_tau<<<dim3((nout + 127) / 128, h->C), 128, 0, h->st>>>(h->Gq, nt, latt_params(h, 1));
    CKL();
  }
  if (!cb) return 0;
  RET(ensure_obs_host(h));
  CK(cudaMemcpyAsync(h->tau_host, h->Gq, 4 * (size_t)h->B * NN * sizeof(zd), cudaMemcpyDeviceToHost, h->st));
  CK(cudaMemcpyAsync(h->phase_host, h->phase, (size_t)h->C * sizeof(zd), cudaMemcpyDeviceToHost, h->st));
  CK(cudaStreamSynchronize(h->st));
  for (int c = 0; c < h->C; ++c)
    cb(ctx, c, nt, 1, h->tau_host + (size_t)c * 4 * h->F * NN * 2, h->phase_host + 2 * c);
  return 0;
}

// ---- CGR2_2 ---------------------------------------------------------------------------------
// Column-pivoted QR (ZGEQP3 semantics, cluster kernel) of the N2 x N2 matrices A in place.
static int qrp_n(alfgpu_s* h, zd* A, int N2, zd* tau, int* jpvt, double* D, double* vn, QRInfo* info) {
  if (h->qr2_mode)  // the row-distributed cluster QR, in place (rows read before any output is written)
    return launch_qrr(h, A, A, N2, h->CL2, h->qr2_mode == 2, h->qr2_ws, tau, jpvt, D, info, nullptr, 0);
  QRParams q;
  memset(&q, 0, sizeof(q));
  q.A = A; q.lda = N2; q.sA = (long long)N2 * N2; q.N = N2;
  q.tau = tau; q.sT = N2; q.jpvt = jpvt; q.sP = N2; q.D = D; q.sD = N2; q.vn = vn; q.sV = 2 * N2;
  q.info = info;
  cudaLaunchConfig_t cfg;
  memset(&cfg, 0, sizeof(cfg));
  cfg.gridDim = dim3(h->CL, h->B, 1);
  cfg.blockDim = dim3(QR_THREADS, 1, 1);
  cfg.dynamicSmemBytes = (size_t)N2 * sizeof(zd);
  cfg.stream = h->st;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = h->CL; at[0].val.clusterDim.y = 1; at[0].val.clusterDim.z = 1;
  cfg.attrs = at; cfg.numAttrs = 1;
  h->launches++;
  CK(cudaLaunchKernelEx(&cfg, k_qrp, q));
  return 0;
}

// Q C for the reflectors of the factored N2 x N2 matrix F (ZUNMQR 'L','N'), all columns of C.
static int unmqr_n(alfgpu_s* h, const zd* F, const zd* tau, zd* Cm, int N2) {
  const long long NN2 = (long long)N2 * N2;
  for (int j0 = ((N2 - 1) / BQR_NB) * BQR_NB; j0 >= 0; j0 -= BQR_NB) {
    const int w = (N2 - j0 < BQR_NB) ? N2 - j0 : BQR_NB;
    BQRApply ap;
    ap.V = F; ap.ldv = N2; ap.sV = NN2; ap.tau = tau; ap.sT = N2;
    ap.C = Cm; ap.ldc = N2; ap.sC = NN2;
    ap.N = N2; ap.j0 = j0; ap.nb = w; ap.c0 = 0; ap.conj_tau = 0; ap.init = 0;
    bqr_apply<ArD>(ap, dim3(N2, h->B), h->st);
    CKL();
  }
  return 0;
}

// CGR2_2, default branch (cgr2_2_mod.F90:317-425) for all (chain, flavour) pairs:
// udv2 = right state (0 -> tau), udv1 = stored left state; results into Hn = GRT0, GR00, GRTT, GR0T.
static int cgr2_2(alfgpu_s* h, const UDVSet& udv2, const UDVSet& udv1) {
  const int N = h->N, B = h->B, N2 = 2 * N;
  const long long NN = (long long)N * N, NN2 = (long long)N2 * N2;
  const dim3 gN((unsigned)((NN + 255) / 256), B), gN2((unsigned)((NN2 + 255) / 256), B);
  // V1^-1 = P R^-1 D^-1 Q^H from the pivoted QR of V1 (INV_C, mymats_mod.F90:546-593)
  RET(qr_any(h, udv1.V, nullptr, h->QRw, 1));
  RET(orgqr_any(h, h->QRw, h->Qt));
  k_scaled_adjoint<<<gN, 256, 0, h->st>>>(h->Qt, h->DUP, h->RHS, N);
  CKL();
  {
    TrsvParams t{};
    t.T = h->QRw; t.ldt = N; t.sT = NN; t.B = h->RHS; t.vstride = N; t.estride = 1; t.sB = NN;
    t.N = N; t.nvec = N; t.lower = 0; t.conj_io = 0;
    prof_begin(h, ALFGPU_PROF_SOLVE);
    RET(trsv(h, t));
    prof_end(h);
    CKL();
  }
  k_perm_rows<<<gN, 256, 0, h->st>>>(h->RHS, h->jpvt, h->V1I, N);
  CKL();
  // HLPB2 / HLPB1 = HLPB2^H, QDRP of HLPB1 (2N x 2N)
  k_cgr22_build<<<gN, 256, 0, h->st>>>(udv1.U, udv1.D, h->V1I, udv2.U, udv2.D, udv2.V, h->HB2, h->HB1, h->first2, N);
  CKL();
  prof_begin(h, ALFGPU_PROF_QR);
  RET(qrp_n(h, h->HB1, N2, h->tau2, h->jpvt2, h->D3, h->vn2, h->info2));
  prof_end(h);
  // solve_extended_System: HLP = P blockdiag, R^H Y = HLP (ZTRSM L,U,C), rows / D3, Q Y (ZUNMQR)
  k_cgr22_hlp<<<gN2, 256, 0, h->st>>>(h->HB2, h->jpvt2, h->HLP, N);
  CKL();
  {
    TrsvParams t{};
    t.T = h->HB1; t.ldt = N2; t.sT = NN2; t.B = h->HLP; t.vstride = N2; t.estride = 1; t.sB = NN2;
    t.N = N2; t.nvec = N2; t.lower = 1; t.conj_io = 0; t.trans = 1;
    t.oscale = nullptr;
    prof_begin(h, ALFGPU_PROF_SOLVE);
    RET(trsv(h, t));
    prof_end(h);
    CKL();
  }
  {
    // HLP(I, :) *= conj(1 / D3(I)): D3 is real
    dim3 grid((unsigned)((NN2 + 255) / 256), B);
    k_scale_rows_inv<<<grid, 256, 0, h->st>>>(h->HLP, h->D3, N2);
    CKL();
  }
  prof_begin(h, ALFGPU_PROF_ORGQR);
  RET(unmqr_n(h, h->HB1, h->tau2, h->HLP, N2));
  prof_end(h);
  k_cgr22_blocks<<<gN, 256, 0, h->st>>>(h->HLP, h->first2, h->Hn[0], h->Hn[1], h->Hn[2], h->Hn[3], N);
  CKL();
  return 0;
}

// TAU_M's propagation products on the tensor-core GEMM (mixed form, real slice scales), in
// place (the operand is sliced before the product overwrites it), with the G wraps' digit count:
// PROPR   X <- diag(S) expT X          (tau_m_mod.F90:213-236)
// PROPRM1 X <- X expTinv diag(Sinv)    (tau_m_mod.F90:238-263)
// With vector vertices (pairblock) the slice's vertex product is applied explicitly after the
// product instead of as a row / column scale.
static bool oz_tau(alfgpu_s* h) { return h->mixed && h->oz && (!h->eexp_complex || h->pairblock); }
static int oz_propr(alfgpu_s* h, zd* X, int nt1) {
  const int N = h->N, B = h->B, S = h->ozw_S;
  const long long NN = (long long)N * N;
  RET(oz_slice(h, X, OZ_CROWS, N, 1, NN, 0, nullptr, 0, N, N, nullptr, S, h->oz_bits, h->oz_Rp2N, h->oz_Kpad,
               h->ozGB, h->ozGBe, B));
  RET(oz_gemm(h, h->tmE[0], h->tmGB, N, 2 * N, h->oz_Kpad, S, h->oz_bits, h->oz_bn, h->oz_nst, h->oz_RpN,
              h->oz_Rp2N, h->F, 0, h->ozEe[0], h->ozGBe, OZ_OUT_COLS, 0, X, 1, N, NN, B,
              h->pairblock ? nullptr : h->S, N, h->oz_S, S));
  return h->pairblock ? vtx_left(h, X, nt1) : 0;
}
static int oz_proprm1(alfgpu_s* h, zd* X, int nt1) {
  const int N = h->N, B = h->B, S = h->ozw_S;
  const long long NN = (long long)N * N;
  RET(oz_slice(h, X, OZ_CROWS, 1, N, NN, 0, nullptr, 0, N, N, nullptr, S, h->oz_bits, h->oz_Rp2N, h->oz_Kpad,
               h->ozGA, h->ozGAe, B));
  RET(oz_gemm(h, h->tmGA, h->tmE[3], 2 * N, N, h->oz_Kpad, S, h->oz_bits, h->oz_bn, h->oz_nst, h->oz_Rp2N,
              h->oz_RpN, 0, h->F, h->ozGAe, h->ozEe[3], OZ_OUT_ROWS, 0, X, 1, N, NN, B, nullptr, 0, S, h->oz_S,
              h->pairblock ? nullptr : h->Sinv, N));
  return h->pairblock ? vtx_right_inv(h, X, nt1) : 0;
}

// TAU_M (tau_m_mod.F90:56-211), finite temperature, after the sweep: GT0, G0T, G00, GTT for
// every slice, ObserT each slice, CGR2_2 and Control_Precision_tau every Nwrap block.
static int tau_m(alfgpu_s* h, alfgpu_obs_cb cb, void* ctx) {
  const int N = h->N, B = h->B, L = h->L, F = h->F;
  const long long NN = (long long)N * N;
  const dim3 gN((unsigned)((NN + 255) / 256), B);
  k_tau_init<<<gN, 256, 0, h->st>>>(h->G, h->G00, h->GT0, h->GTT, h->G0T, N);
  CKL();
  RET(obs_tau(h, cb, ctx, 0));
  RET(udv_reset(h, h->udvr_tau));
  int NST = 1;
  for (int NT = 0; NT < L; ++NT) {
    const int NT1 = NT + 1;
    const bool pb = h->pairblock;
    if (!pb) RET(slice_scale(h, NT1));
    prof_begin(h, ALFGPU_PROF_HOP);
    if (h->cb) {  // PROPR X <- P B_T X, PROPRM1 X <- X B_T^-1 P^-1 with the bond operators
      zd* Xs[3] = {h->GT0, h->G0T, h->GTT};
      for (int k = 0; k < 3; ++k) {
        if (k >= 1) {  // PROPRM1 (G0T, then the first half of GTT)
          RET(cb_apply(h, Xs[k], CB_MMTHL_M1));
          if (pb) RET(vtx_right_inv(h, Xs[k], NT1));
          else RET(scale_rc(h, Xs[k], nullptr, 0, h->Sinv));
        }
        if (k != 1) {  // PROPR (GT0, then the second half of GTT)
          RET(cb_apply(h, Xs[k], CB_MMTHR));
          if (pb) RET(vtx_left(h, Xs[k], NT1));
          else RET(scale_rc(h, Xs[k], h->S, 0, nullptr));
        }
      }
    } else if (oz_tau(h)) {
      RET(oz_propr(h, h->GT0, NT1));     // PROPR(GT0)
      RET(oz_proprm1(h, h->G0T, NT1));   // PROPRM1(G0T)
      RET(oz_proprm1(h, h->GTT, NT1));   // PROPRM1 then PROPR (GTT)
      RET(oz_propr(h, h->GTT, NT1));
    } else {
    {  // PROPR(GT0): GT0 = S (expT GT0)
      GemmParams p = gsq(h, B);
      p.A = h->expT; p.realA = 1; p.modA = F; p.B = h->GT0; p.C = h->T1;
      if (!pb) { p.rs = h->S; p.sRS = N; }
      RET(gemm(h, p));
      std::swap(h->GT0, h->T1);
      if (pb) RET(vtx_left(h, h->GT0, NT1));
    }
    {  // PROPRM1(G0T): G0T = (G0T expTinv) Sinv
      GemmParams p = gsq(h, B);
      p.A = h->G0T; p.B = h->expTinv; p.realB = 1; p.modB = F; p.C = h->T1;
      if (!pb) { p.cs = h->Sinv; p.sCS = N; }
      RET(gemm(h, p));
      std::swap(h->G0T, h->T1);
      if (pb) RET(vtx_right_inv(h, h->G0T, NT1));
    }
    {  // PROPRM1 then PROPR (GTT): GTT = S expT (GTT expTinv Sinv)
      GemmParams p = gsq(h, B);
      p.A = h->GTT; p.B = h->expTinv; p.realB = 1; p.modB = F; p.C = h->T1;
      if (!pb) { p.cs = h->Sinv; p.sCS = N; }
      RET(gemm(h, p));
      if (pb) RET(vtx_right_inv(h, h->T1, NT1));
      GemmParams q = gsq(h, B);
      q.A = h->expT; q.realA = 1; q.modA = F; q.B = h->T1; q.C = h->GTT;
      if (!pb) { q.rs = h->S; q.sRS = N; }
      RET(gemm(h, q));
      if (pb) RET(vtx_left(h, h->GTT, NT1));
    }
    }
    prof_end(h);
    RET(obs_tau(h, cb, ctx, NT1));
    if (NST <= h->Nstm && NT1 == h->stab_nt[NST]) {
      RET(wrapur_u(h, h->udvr_tau, h->stab_nt[NST - 1], NT1));
      RET(cgr2_2(h, h->udvr_tau, h->udvst[NST - 1]));
      // Control_Precision_tau: G vs new G00, old GTT / GT0 / G0T vs new
      zd* olds[4] = {h->GT0, h->G, h->GTT, h->G0T};
      for (int k = 0; k < 4; ++k) {
        CK(cudaMemsetAsync(h->cmp_tau + 2ll * k * B, 0, 2 * (size_t)B * sizeof(double), h->st));
        k_compare<<<dim3(CMP_BLOCKS, B), 256, 0, h->st>>>(h->Hn[k], olds[k], N, h->cmp_tau + 2ll * k * B, h->err);
        CKL();
      }
      k_tau_stats<<<(h->C + 127) / 128, 128, 0, h->st>>>(h->cmp_tau, h->C, F, h->stat);
      CKL();
      std::swap(h->GT0, h->Hn[0]);
      std::swap(h->G00, h->Hn[1]);
      std::swap(h->GTT, h->Hn[2]);
      std::swap(h->G0T, h->Hn[3]);
      NST++;
    }
  }
  return 0;
}

// Hopping wraps with the slice's deferred vertex scalings (Wrapgr_mod.F90:110-114, 237-241).
// up:   G <- expT (S G Sinv) expTinv      down: G <- expTinv (Sinv G S) expT
static int hop_impl(alfgpu_s* h, int up, int with_scale);
static int hop(alfgpu_s* h, int up, int with_scale) {
  prof_begin(h, ALFGPU_PROF_HOP);
  int r = hop_impl(h, up, with_scale);
  prof_end(h);
  return r;
}
static int hop_impl(alfgpu_s* h, int up, int with_scale) {
  const int N = h->N, F = h->F, B = h->B;
  if (h->cb) {  // WRAPGRUP: mmthr, mmthl_m1; WRAPGRDO: mmthl, mmthr_m1 (bond passes, both forms)
    if (with_scale) RET(scale_rc(h, h->G, up ? h->S : h->Sinv, 0, up ? h->Sinv : h->S));
    RET(cb_apply(h, h->G, up ? CB_MMTHR : CB_MMTHL));
    return cb_apply(h, h->G, up ? CB_MMTHL_M1 : CB_MMTHR_M1);
  }
  if (h->mixed && h->oz && !(with_scale && h->eexp_complex)) {
    // up:   T1 = expT diag(S) G (row-major), G = T1 diag(Sinv) expTinv
    // down: T1 = G diag(S) expT (column-major), G = expTinv diag(Sinv) T1
    // the wraps use the first ozw_S digit slices (the expT slices hold oz_S per flavour)
    const long long NN = (long long)N * N;
    const int S = h->ozw_S, SE = h->oz_S, bits = h->oz_bits, Kp = h->oz_Kpad, RpN = h->oz_RpN, Rp2 = h->oz_Rp2N;
    const int bn = h->oz_bn, nst = h->oz_nst;
    const zd* s1 = with_scale ? h->S : nullptr;
    const zd* s2 = with_scale ? h->Sinv : nullptr;
    if (up) {
      RET(oz_slice(h, h->G, OZ_CROWS, N, 1, NN, 0, s1, N, N, N, nullptr, S, bits, Rp2, Kp, h->ozGB, h->ozGBe, B));
      RET(oz_gemm(h, h->tmE[0], h->tmGB, N, 2 * N, Kp, S, bits, bn, nst, RpN, Rp2, F, 0, h->ozEe[0], h->ozGBe,
                  OZ_OUT_COLS, 0, h->T1, N, 1, NN, B, nullptr, 0, SE, S));
      RET(oz_slice(h, h->T1, OZ_CROWS, N, 1, NN, 0, s2, N, N, N, nullptr, S, bits, Rp2, Kp, h->ozGA, h->ozGAe, B));
      RET(oz_gemm(h, h->tmGA, h->tmE[3], 2 * N, N, Kp, S, bits, bn, nst, Rp2, RpN, 0, F, h->ozGAe, h->ozEe[3],
                  OZ_OUT_ROWS, 0, h->G, 1, N, NN, B, nullptr, 0, S, SE));
    } else {
      RET(oz_slice(h, h->G, OZ_CROWS, 1, N, NN, 0, s1, N, N, N, nullptr, S, bits, Rp2, Kp, h->ozGA, h->ozGAe, B));
      RET(oz_gemm(h, h->tmGA, h->tmE[2], 2 * N, N, Kp, S, bits, bn, nst, Rp2, RpN, 0, F, h->ozGAe, h->ozEe[2],
                  OZ_OUT_ROWS, 0, h->T1, 1, N, NN, B, nullptr, 0, S, SE));
      RET(oz_slice(h, h->T1, OZ_CROWS, N, 1, NN, 0, s2, N, N, N, nullptr, S, bits, Rp2, Kp, h->ozGB, h->ozGBe, B));
      RET(oz_gemm(h, h->tmE[1], h->tmGB, N, 2 * N, Kp, S, bits, bn, nst, RpN, Rp2, F, 0, h->ozEe[1], h->ozGBe,
                  OZ_OUT_COLS, 0, h->G, 1, N, NN, B, nullptr, 0, SE, S));
    }
    return 0;
  }
  if (h->mixed) {
    const double* E1 = up ? h->expT : h->expTinv;
    const double* E2 = up ? h->expTinv : h->expT;
    if (up) {
      GemmParams p = gsq(h, B);
      p.A = E1; p.modA = F; p.B = h->G; p.C = h->T1;
      if (with_scale) { p.ks = h->S; p.sKS = N; p.ksOnA = 0; }
      RET(gemm32(h, p, ST_R64, ST_C128, ST_C128));
      GemmParams q = gsq(h, B);
      q.A = h->T1; q.B = E2; q.modB = F; q.C = h->G;
      if (with_scale) { q.ks = h->Sinv; q.sKS = N; q.ksOnA = 1; }
      RET(gemm32(h, q, ST_C128, ST_R64, ST_C128));
    } else {
      GemmParams p = gsq(h, B);
      p.A = h->G; p.B = E2; p.modB = F; p.C = h->T1;
      if (with_scale) { p.ks = h->S; p.sKS = N; p.ksOnA = 1; }
      RET(gemm32(h, p, ST_C128, ST_R64, ST_C128));
      GemmParams q = gsq(h, B);
      q.A = E1; q.modA = F; q.B = h->T1; q.C = h->G;
      if (with_scale) { q.ks = h->Sinv; q.sKS = N; q.ksOnA = 0; }
      RET(gemm32(h, q, ST_R64, ST_C128, ST_C128));
    }
    return 0;
  }
  const double* E1 = up ? h->expT : h->expTinv;   // left factor
  const double* E2 = up ? h->expTinv : h->expT;   // right factor
  if (up) {
    // T1 = expT * diag(S) * G ; G = T1 * diag(Sinv) * expTinv
    GemmParams p = gsq(h, B);
    p.A = E1; p.realA = 1; p.modA = F;
    p.B = h->G; p.C = h->T1;
    if (with_scale) { p.ks = h->S; p.sKS = N; p.ksOnA = 0; }
    RET(gemm(h, p));
    GemmParams q = gsq(h, B);
    q.A = h->T1; q.B = E2; q.realB = 1; q.modB = F; q.C = h->G;
    if (with_scale) { q.ks = h->Sinv; q.sKS = N; q.ksOnA = 1; }
    RET(gemm(h, q));
  } else {
    // T1 = G * diag(S) * expT ; G = expTinv * diag(Sinv) * T1
    GemmParams p = gsq(h, B);
    p.A = h->G; p.B = E2; p.realB = 1; p.modB = F; p.C = h->T1;
    if (with_scale) { p.ks = h->S; p.sKS = N; p.ksOnA = 1; }
    RET(gemm(h, p));
    GemmParams q = gsq(h, B);
    q.A = E1; q.realA = 1; q.modA = F; q.B = h->T1; q.C = h->G;
    if (with_scale) { q.ks = h->Sinv; q.sKS = N; q.ksOnA = 0; }
    RET(gemm(h, q));
  }
  return 0;
}

// Metropolis updates of one slice in blocks of kblk visits, each followed by its flush.
// The slice's delayed-update blocks.  Per block: the Metropolis visits (k_update), the flush
// operands (k_flush_xy) and the flush G -= X Y.  With h->overlap (no vector vertices, no phase
// profile) the visits of block k + 1 run on the second stream while the flush of block k runs on
// st: before the flush, k_sub_gather snapshots G over block k + 1's positions, and k_sub_stage
// applies block k's updates to that snapshot (the same Woodbury form), so block k + 1 starts from
// its submatrix without waiting for the full-matrix flush.  The rank array m is kept per block
// parity because the flush of block k reads it while block k + 1 writes its own.
static int update_slice(alfgpu_s* h, int nt1, int dir, int visit_base, const double* draws_dev) {
  const int N = h->N, F = h->F, M = h->M;
  const long long NN = (long long)N * N;
  const size_t nblk = h->blk_start[dir].size();
  // the overlap needs room on the SMs next to the flush: the default tensor-core flush tiles fill
  // them (one CTA per SM by shared memory and TMEM), the paired tiles leave room for k_update
  const bool ozf = h->mixed && h->oz && !h->oz_narrow && !(h->d.reserved[0] & ALFGPU_FLAG_DF_FLUSH);
  const bool ov = h->overlap && (!ozf || h->ozf_pairs) && !h->pairblock && !h->profiling && nblk > 1;
  const bool dfv = h->mixed && !(h->d.reserved[0] & ALFGPU_FLAG_FP64_VISITS);  // visits in double-float
  const long long msz = (long long)h->C + h->B;
  VertexDev V;
  V.site = h->v_site; V.site2 = h->v_site2; V.nsite = h->v_nsite; V.type = h->v_type; V.sK = (long long)F * M;
  if (ov) {  // the slice's G is ready on st: the first block's visits may start on st2
    CK(cudaEventRecord(h->ev_fork, h->st));
    CK(cudaStreamWaitEvent(h->st2, h->ev_fork, 0));
  }
  for (size_t blk = 0; blk < nblk; ++blk) {
    int* mb = h->m + (ov ? (long long)(blk & 1) * msz : 0);
    cudaStream_t su = ov ? h->st2 : h->st;
    if (ov && blk > 0) {  // block blk's submatrix after block blk - 1's updates
      // FP64 in both forms: this submatrix is the block's G0, whose Gamma^-1 sets the next flush
      // (double-float here raised the mixed form's largest Precision Green from 9e-6 to 6e-5)
      const int* mprev = h->m + (long long)((blk - 1) & 1) * msz;
      const dim3 gs((UPD_KMAX + 7) / 8, h->B), bs(32, 8);
      k_sub_stage<ArD><<<gs, bs, 0, su>>>(h->Gsnap, h->posn, h->npos, mprev, N, F, h->X, h->Y, h->Gsub);
      CKL();
    }
    UpdParams u;
    memset(&u, 0, sizeof(u));
    u.N = N; u.F = F; u.M = M; u.L = h->L; u.NSUN = h->NSUN;
    u.nt1 = nt1; u.dir = dir; u.q0 = h->blk_start[dir][blk]; u.nq = h->blk_cnt[dir][blk];
    u.visit_base = visit_base;
    u.nChains = h->C;
    u.G = h->G; u.sG = F * NN;
    u.V.site = h->v_site; u.V.site2 = h->v_site2; u.V.nsite = h->v_nsite; u.V.type = h->v_type;
    u.V.sK = (long long)F * M;
    u.tab = h->v_tab;
    u.fields = h->fields;
    u.draws = draws_dev; u.sDraws = 6ll * M * h->L;
    u.rngkey = h->rngkey; u.rngctr = h->rngctr;
    u.phase = h->phase; u.m_out = mb; u.W = h->W; u.sites_out = h->sites; u.delta_out = h->dlt; u.cnt = h->cnt;
    u.Gsub = (ov && blk > 0) ? h->Gsub : nullptr;
    if (h->recording) { u.rec_acc = h->rec_acc; u.rec_ratio = h->rec_ratio; u.sRec = 2ll * M * h->L; }
    u.ft = h->ft;
    if (h->pairblock) {
      u.vsite2 = h->v_blk2; u.vcoef = h->v_vc; u.sites2_out = h->sites2_out; u.coef_out = h->coef_out;
    }
    prof_begin(h, ALFGPU_PROF_UPDATE);
    if (dfv) k_update<ArF><<<h->C, UPD_THREADS, upd_smem_bytes(), su>>>(u);
    else k_update<ArD><<<h->C, UPD_THREADS, upd_smem_bytes(), su>>>(u);
    prof_end(h);
    CKL();
    if (ov) {  // the flush operands need this block's decisions (and the previous flush, on st)
      CK(cudaEventRecord(h->ev_join, h->st2));
      CK(cudaStreamWaitEvent(h->st, h->ev_join, 0));
    }
    prof_begin(h, ALFGPU_PROF_FLUSH);
    const int* s2o = h->pairblock ? h->sites2_out : nullptr;
    const double* co = h->pairblock ? h->coef_out : nullptr;
    if (dfv)
      k_flush_xy<ArF><<<dim3((N + 7) / 8, h->B), dim3(32, 8), 0, h->st>>>(h->G, F * NN, N, F, mb, h->sites, h->W,
                                                                         h->X, h->Y, s2o, co);
    else
      k_flush_xy<ArD><<<dim3((N + 7) / 8, h->B), dim3(32, 8), 0, h->st>>>(h->G, F * NN, N, F, mb, h->sites, h->W,
                                                                         h->X, h->Y, s2o, co);
    CKL();
    if (ov && blk + 1 < nblk) {  // snapshot for the next block, then let its visits start
      k_sub_gather<<<h->B, 256, 0, h->st>>>(h->G, F * NN, N, F, M, V, dir, h->blk_start[dir][blk + 1],
                                            h->blk_cnt[dir][blk + 1], h->Gsnap, h->posn, h->npos);
      CKL();
      CK(cudaEventRecord(h->ev_fork, h->st));
      CK(cudaStreamWaitEvent(h->st2, h->ev_fork, 0));
    }
    void* Gst = h->G;
    void* Xst = h->X;
    void* Yst = h->Y;
    // G -= X Y, rank m per chain
    GemmParams p = gemm_defaults();
    p.m = N; p.n = N; p.k = UPD_KMAX;
    p.A = Xst; p.lda = N; p.sA = (long long)N * UPD_KMAX;
    p.B = Yst; p.ldb = UPD_KMAX; p.sB = (long long)N * UPD_KMAX;
    p.C = (zd*)Gst; p.ldc = N; p.sC = NN;
    p.alpha = zmk(-1.0, 0.0); p.beta = zmk(1.0, 0.0);
    p.batch = h->B;
    // X / Y keep two flavour slots per chain; per-batch rank K = m[chain]
    if (F == 1) { p.sA = 2ll * N * UPD_KMAX; p.sB = 2ll * N * UPD_KMAX; }
    p.kdyn = mb + h->C;  // per-(chain, flavour) rank, written by k_update
    if (ozf) {
      // G -= X Y as one real product: [Re X | Im X] times the K-doubled complex rows of Y
      const int Kf = 2 * UPD_KMAX;
      RET(oz_slice(h, h->X, OZ_CKA, 1, N, p.sA, 0, nullptr, 0, N, UPD_KMAX, p.kdyn, h->ozf_S, h->ozf_bits,
                   h->oz_RpN, Kf, h->ozXA, h->ozXAe, h->B));
      RET(oz_slice(h, h->Y, OZ_CKB, UPD_KMAX, 1, p.sB, 0, nullptr, 0, N, UPD_KMAX, p.kdyn, h->ozf_S, h->ozf_bits,
                   h->oz_Rp2N, Kf, h->ozYB, h->ozYBe, h->B));
      RET(oz_gemm(h, h->tmXA, h->tmYB, N, 2 * N, Kf, h->ozf_S, h->ozf_bits, h->ozf_bn, h->ozf_nst, h->oz_RpN,
                  h->oz_Rp2N, 0, 0, h->ozXAe, h->ozYBe, OZ_OUT_COLS, 1, h->G, 1, N, NN, h->B, nullptr, 0, 0, 0,
                  nullptr, 0, h->ozf_grid));
    } else if (h->mixed) RET(gemm32(h, p, ST_C128, ST_C128, ST_C128));
    else RET(gemm(h, p));
    prof_end(h);
    // a phase ends with this block: its vertex wraps, explicit (up pass: E(s_old) G E(s_old)^-1 with
    // the fields before the slice's updates; down pass: E(s_new)^-1 G E(s_new))
    const int ph = h->pairblock ? h->blk_phase_end[dir][blk] : -1;
    if (ph >= 0) {
      prof_begin(h, ALFGPU_PROF_HOP);
      if (dir == 0) {
        RET(vtx_phase(h, h->G, ph, nt1, true, 0, 0, true));
        RET(vtx_phase(h, h->G, ph, nt1, true, 1, 0, false));
      } else {
        RET(vtx_phase(h, h->G, ph, nt1, false, 1, 0, true));
        RET(vtx_phase(h, h->G, ph, nt1, false, 0, 0, false));
      }
      prof_end(h);
    }
  }
  return 0;
}

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------
extern "C" {

const char* alfgpu_error_string(int code) {
  switch (code) {
    case ALFGPU_ERROR_NONE: return "no error";
    case ALFGPU_ERROR_GENERIC: return "generic error";
    case ALFGPU_ERROR_UNSTABLE_MATRIX: return "Precision Green exceeds 10: unstable calculation";
    case ALFGPU_ERROR_FIELDS: return "invalid field values";
    case ALFGPU_ERROR_HAMILTONIAN: return "invalid operator tables";
    case ALFGPU_ERROR_CUDA: return "CUDA runtime error";
    case ALFGPU_ERROR_ARGUMENT: return "invalid argument";
    case ALFGPU_ERROR_UNSUPPORTED: return "model feature not supported on the GPU path";
    case ALFGPU_ERROR_NAN: return "NaN in the Green function";
    case ALFGPU_ERROR_TIMEOUT: return "device wait timed out";
    case ALFGPU_ERROR_SIZE: return "Ndim exceeds the static scratch of the no-allocation entry point";
    default: return "unknown error";
  }
}

// Buffers, tensor maps and tile shapes of the tensor-core GEMMs of the mixed form; leaves
// h->oz = 0 (double-float GEMMs) when a size does not fit.
static int oz_setup(alfgpu_s* h) {
  const int N = h->N;
  const size_t B = h->B, F = h->F;
  h->oz = 0;
  h->oz_Kpad = oz_round(N, OZ_KC);
  h->oz_RpN = oz_round(N, OZ_BM);
  h->oz_Rp2N = oz_round(2 * N, OZ_BM);
  if (oz_pick(h->oz_Kpad, &h->oz_bits, &h->oz_S) || oz_pick(2 * UPD_KMAX, &h->ozf_bits, &h->ozf_S)) return 0;
  // digit slices of the G wraps / TAU_M propagation (reserved[1]) and the UDV propagation
  // (reserved[2]): the target bits rounded up to whole slices, at most oz_S
  auto slices_for = [&](int target) {
    if (target <= 0) return h->oz_S;
    const int s = (target + h->oz_bits - 1) / h->oz_bits;
    return std::max(2, std::min(h->oz_S, s));
  };
  h->ozw_S = slices_for(h->d.reserved[1]);
  h->ozp_S = slices_for(h->d.reserved[2]);
  // CTAs of one wrap product at BN = 32; fewer than two per SM: the narrow tile
  int nsm = 152;
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, h->dev);
  const long long tiles = (long long)((N + OZ_BM - 1) / OZ_BM) * ((2 * N + 31) / 32) * (long long)B;
  const int narrow = tiles < 2ll * nsm && !(h->d.reserved[0] & ALFGPU_FLAG_TENSOR_WIDE);
  h->oz_narrow = narrow;
  if (oz_pick_tile(h->oz_S, h->oz_Kpad / OZ_KC, &h->oz_bn, &h->oz_nst,
                   narrow || (h->d.reserved[0] & ALFGPU_FLAG_OZ_DEEP_RING)) ||
      oz_pick_tile(h->ozf_S, 2 * UPD_KMAX / OZ_KC, &h->ozf_bn, &h->ozf_nst, narrow))
    return 0;
  if (!narrow && (h->d.reserved[0] & ALFGPU_FLAG_OZ_FLUSH_RESIDENT)) {
    // K = 64 products as persistent CTAs, one per SM, that keep a tile's A digit slices in a ring
    // of S stages and reuse them for the following tiles of the same M-tile
    if (oz_smem_bytes(32, h->ozf_S, 1, h->ozf_S) <= 227 * 1024) {
      h->ozf_bn = 32;
      h->ozf_nst = h->ozf_S;
      h->ozf_grid = nsm;
    }
  } else if (!narrow && !(h->d.reserved[0] & ALFGPU_FLAG_OZ_FLUSH_SINGLE)) {
    // K = 64 products (flush, compact-WY update) on 16-wide tiles with a ring small enough for
    // two CTAs per SM ((S + 1) x 16 TMEM columns round to 256 of the SM's 512) and room beside
    // them for one k_update CTA, so the next block's visits can overlap the flush
    int st = 8;
    while (st > 2 && 2 * oz_smem_bytes(16, h->ozf_S, 1, st) + upd_smem_bytes() + 16 * 1024 > 227 * 1024) --st;
    h->ozf_bn = 16;
    h->ozf_nst = st;
    h->ozf_pairs = 1;
    h->ozf_grid = 2 * nsm;  // more CTAs would take the room beside them (TMEM is not a launch resource)
  }
  if (!oz_encoder()) return 0;
  const size_t S = h->oz_S, Sf = h->ozf_S, Kp = h->oz_Kpad, Kf = 2 * UPD_KMAX, RpN = h->oz_RpN, Rp2 = h->oz_Rp2N;
  int r = 0;
  for (int a = 0; a < 4; ++a) { r |= dalloc(h, &h->ozE[a], F * S * RpN * Kp); r |= dalloc(h, &h->ozEe[a], F * RpN); }
  r |= dalloc(h, &h->ozGA, B * S * Rp2 * Kp); r |= dalloc(h, &h->ozGAe, B * Rp2);
  r |= dalloc(h, &h->ozGB, B * S * Rp2 * Kp); r |= dalloc(h, &h->ozGBe, B * Rp2);
  r |= dalloc(h, &h->ozXA, B * Sf * RpN * Kf); r |= dalloc(h, &h->ozXAe, B * RpN);
  r |= dalloc(h, &h->ozYB, B * Sf * Rp2 * Kf); r |= dalloc(h, &h->ozYBe, B * Rp2);
  r |= dalloc(h, &h->ozGm, B * 1024); r |= dalloc(h, &h->ozTm, B * 1024);
  r |= dalloc(h, &h->ozWm, B * 32 * (size_t)N); r |= dalloc(h, &h->ozXm, B * 32 * (size_t)N);
  if (r) return ALFGPU_ERROR_CUDA;
  int t = 0;
  for (int a = 0; a < 4; ++a)
    t |= oz_tmap(&h->tmE[a], h->ozE[a], (int)Kp, (long long)(F * S * RpN), a < 2 ? OZ_BM : h->oz_bn);
  t |= oz_tmap(&h->tmGA, h->ozGA, (int)Kp, (long long)(B * S * Rp2), OZ_BM);
  t |= oz_tmap(&h->tmGB, h->ozGB, (int)Kp, (long long)(B * S * Rp2), h->oz_bn);
  t |= oz_tmap(&h->tmXA, h->ozXA, (int)Kf, (long long)(B * Sf * RpN), OZ_BM);
  t |= oz_tmap(&h->tmYB, h->ozYB, (int)Kf, (long long)(B * Sf * Rp2), h->ozf_bn);
  if (t) return 0;
  const size_t sm1 = oz_smem_bytes(h->oz_bn, h->oz_S, h->oz_Kpad / OZ_KC, h->oz_nst);
  const size_t sm2 = oz_smem_bytes(h->ozf_bn, h->ozf_S, 1, h->ozf_nst);
  const int sm32 = (int)std::max(h->oz_bn == 32 ? sm1 : 0, h->ozf_bn == 32 ? sm2 : 0);
  const int sm16 = (int)std::max(h->oz_bn == 16 ? sm1 : 0, h->ozf_bn == 16 ? sm2 : 0);
  if (sm32 && (raise_smem_limit(k_oz_gemm<32>, (size_t)sm32) != cudaSuccess ||
               raise_smem_limit(k_oz_gemm<32, true>, (size_t)sm32) != cudaSuccess))
    return ALFGPU_ERROR_CUDA;
  if (sm16 && (raise_smem_limit(k_oz_gemm<16>, (size_t)sm16) != cudaSuccess ||
               raise_smem_limit(k_oz_gemm<16, true>, (size_t)sm16) != cudaSuccess))
    return ALFGPU_ERROR_CUDA;
  if (h->ozf_pairs) {
    // the paired flush CTAs and the overlapped k_update CTA share an SM only if the SM is set up
    // with its largest shared-memory carveout while the flush runs
    if (cudaFuncSetAttribute(k_oz_gemm<16, true>, cudaFuncAttributePreferredSharedMemoryCarveout,
                             cudaSharedmemCarveoutMaxShared) != cudaSuccess ||
        cudaFuncSetAttribute(k_update<ArF>, cudaFuncAttributePreferredSharedMemoryCarveout,
                             cudaSharedmemCarveoutMaxShared) != cudaSuccess ||
        cudaFuncSetAttribute(k_update<ArD>, cudaFuncAttributePreferredSharedMemoryCarveout,
                             cudaSharedmemCarveoutMaxShared) != cudaSuccess)
      return ALFGPU_ERROR_CUDA;
  }
  h->oz = 1;
  return 0;
}

int alfgpu_create(alfgpu_t** out, const alfgpu_dims* dims) {
  if (!out || !dims) return ALFGPU_ERROR_ARGUMENT;
  *out = nullptr;
  const alfgpu_dims& d = *dims;
  if (d.ndim < 1 || d.ndim > 4096 || d.n_fl < 1 || d.n_fl > 2 || d.n_sun < 1 || d.n_op < 1 || d.ltrot < 1 ||
      d.nwrap < 1 || d.n_chains < 1)
    return ALFGPU_ERROR_ARGUMENT;
  if (d.precision != ALFGPU_PRECISION_FP64 && d.precision != ALFGPU_PRECISION_MIXED) return ALFGPU_ERROR_ARGUMENT;
  if (d.ltau != 0 && d.ltau != 1) return ALFGPU_ERROR_ARGUMENT;
  if ((d.reserved[0] & ALFGPU_FLAG_QR_HALF_CLUSTER) && (d.reserved[0] & ALFGPU_FLAG_QR_FULL_CLUSTER))
    return ALFGPU_ERROR_ARGUMENT;
  if (d.ltau && 2 * d.ndim > 32 * BQR_LROWS) return ALFGPU_ERROR_UNSUPPORTED;  // CGR2_2's 2N-row apply
  alfgpu_s* h = new alfgpu_s();
  h->d = d;
  h->N = d.ndim; h->F = d.n_fl; h->M = d.n_op; h->L = d.ltrot; h->C = d.n_chains; h->B = d.n_chains * d.n_fl;
  h->NSUN = d.n_sun;
  h->Nstm = (d.ltrot % d.nwrap == 0) ? d.ltrot / d.nwrap : d.ltrot / d.nwrap + 1;
  h->stab_nt.resize(h->Nstm + 1);
  h->stab_nt[0] = 0;
  for (int n = 1; n < h->Nstm; ++n) h->stab_nt[n] = d.nwrap * n;
  h->stab_nt[h->Nstm] = d.ltrot;
  h->CL = cluster_size(h->N);
  h->kblk = (d.delay_k > 0 && d.delay_k <= UPD_KMAX) ? d.delay_k : UPD_KMAX;
  h->dev = d.device;
  h->mixed = d.precision == ALFGPU_PRECISION_MIXED;
  h->mixed_propagate = h->mixed && (d.reserved[0] & ALFGPU_FLAG_DF_PROPAGATION);
  {
    const int fl = d.reserved[0];
    const bool force = fl & ALFGPU_FLAG_EXACT_QRP;
    h->exact_dec = force || !(fl & ALFGPU_FLAG_NORM_PIVOT_DECOMPOSE);
    h->exact_cgr = force || !(fl & ALFGPU_FLAG_NORM_PIVOT_CGR);
  }
  h->df_stab = h->mixed && (d.reserved[0] & ALFGPU_FLAG_DF_STAB_GEMM);
  h->df_qr = h->mixed && (d.reserved[0] & ALFGPU_FLAG_DF_STAB_QR);
  h->use_graph = !(d.reserved[0] & ALFGPU_FLAG_NO_GRAPH);
  fill_tables(h->ft);
  auto fail = [&](int code) { alfgpu_destroy(h); return code; };
  if (cudaSetDevice(d.device) != cudaSuccess) return fail(ALFGPU_ERROR_CUDA);
  if (cudaStreamCreateWithFlags(&h->st, cudaStreamNonBlocking) != cudaSuccess ||
      cudaStreamCreateWithFlags(&h->st2, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreateWithFlags(&h->ev_fork, cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&h->ev_join, cudaEventDisableTiming) != cudaSuccess)
    return fail(ALFGPU_ERROR_CUDA);
  h->overlap = !(d.reserved[0] & ALFGPU_FLAG_NO_OVERLAP);
  if (h->CL > 8) {
    if (cudaFuncSetAttribute(k_qrp, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) != cudaSuccess ||
        cudaFuncSetAttribute(k_orgqr, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) != cudaSuccess ||
        cudaFuncSetAttribute(k_bqr_panel, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) != cudaSuccess)
      return fail(ALFGPU_ERROR_CUDA);
  }
  if (raise_smem_limit(k_update<ArD>, upd_smem_bytes()) != cudaSuccess ||
      raise_smem_limit(k_update<ArF>, upd_smem_bytes()) != cudaSuccess)
    return fail(ALFGPU_ERROR_CUDA);
  // shrink the QR cluster until at least one cluster fits on the device
  while (h->CL > 1) {
    cudaLaunchConfig_t cfg;
    memset(&cfg, 0, sizeof(cfg));
    cfg.gridDim = dim3(h->CL, 1, 1);
    cfg.blockDim = dim3(QR_THREADS, 1, 1);
    cfg.dynamicSmemBytes = (size_t)h->N * sizeof(zd);
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = h->CL; at[0].val.clusterDim.y = 1; at[0].val.clusterDim.z = 1;
    cfg.attrs = at; cfg.numAttrs = 1;
    int n1 = 0, n2 = 0;
    int n3 = 0;
    cudaLaunchConfig_t cfg3 = cfg;
    cfg3.dynamicSmemBytes = 0;
    if (cudaOccupancyMaxActiveClusters(&n1, k_qrp, &cfg) == cudaSuccess &&
        cudaOccupancyMaxActiveClusters(&n2, k_orgqr, &cfg) == cudaSuccess &&
        cudaOccupancyMaxActiveClusters(&n3, k_bqr_panel, &cfg3) == cudaSuccess && n1 > 0 && n2 > 0 && n3 > 0)
      break;
    cudaGetLastError();
    h->CL /= 2;
  }
  // exact pivoting on the row-distributed cluster kernel when its row block fits in shared memory.
  // A launch over B matrices whose full-size clusters would put more than two CTAs on every SM
  // takes clusters of CL / 2 CTAs: the same FP64 work in half as many CTAs, each pivot step's
  // cluster exchange and barriers shared by half as many (16 chains of the 16x16 Hubbard model:
  // 512 -> 256 CTAs on 152 SMs, QR time per sweep 501 -> 478 ms).  A grid that fits keeps CL.
  // Rows that do not fit shared memory (N_dim above ~420, CGR2_2's 2N system) stay in a global
  // workspace per CTA (mode 2) instead of falling back to the column-distributed k_qrp.
  h->CLr = h->CL;
  h->qrr_ok = qrr_plan(h->N, h->CL, h->B, d.reserved[0], h->dev, &h->CLr);
  if (d.ltau) h->qr2_mode = qrr_plan(2 * d.ndim, cluster_size(2 * d.ndim), h->B, d.reserved[0], h->dev, &h->CL2);
  // the blocked QR keeps at most BQR_ROWS panel rows per CTA and BQR_LROWS rows per lane
  if (h->N > 32 * BQR_LROWS || (h->N + h->CL - 1) / h->CL > BQR_ROWS) h->exact_dec = h->exact_cgr = 1;
  const size_t N = h->N, NN = N * N, B = h->B, C = h->C, F = h->F, M = h->M, L = h->L;
  int r = 0;
  r |= dalloc(h, &h->expT, F * NN); r |= dalloc(h, &h->expTinv, F * NN);
  r |= dalloc(h, &h->v_site, C * F * M); r |= dalloc(h, &h->v_g, C * F * M); r |= dalloc(h, &h->v_alpha, C * F * M);
  r |= dalloc(h, &h->v_E, C * F * M); r |= dalloc(h, &h->v_type, C * F * M); r |= dalloc(h, &h->v_Eexp, C * F * M * 10);
  r |= dalloc(h, &h->v_site2, C * F * M); r |= dalloc(h, &h->v_nsite, C * F * M);
  r |= dalloc(h, &h->v_kind, C * F * M); r |= dalloc(h, &h->v_blk2, C * F * M); r |= dalloc(h, &h->v_vc, 2 * C * F * M);
  r |= dalloc(h, &h->sites2_out, C * UPD_KMAX); r |= dalloc(h, &h->coef_out, 2 * C * UPD_KMAX);
  r |= dalloc(h, &h->fields_old, C * M);
  r |= dalloc(h, &h->v_tab, C * F * M * 15);
  r |= dalloc(h, &h->v_sptr, C * F * (N + 1)); r |= dalloc(h, &h->v_slist, C * F * 2 * M);
  r |= dalloc(h, &h->fields, C * L * M);
  r |= dalloc(h, &h->G, B * NN); r |= dalloc(h, &h->Gw, B * NN); r |= dalloc(h, &h->T1, B * NN);
  r |= dalloc(h, &h->S, B * N); r |= dalloc(h, &h->Sinv, B * N);

  auto mk_udv = [&](UDVSet& s) {
    int q = 0;
    q |= dalloc(h, &s.U, B * NN); q |= dalloc(h, &s.V, B * NN); q |= dalloc(h, &s.D, B * N); q |= dalloc(h, &s.detU, B);
    return q;
  };
  r |= mk_udv(h->udvl); r |= mk_udv(h->udvr);
  h->udvst.resize(h->Nstm);
  for (auto& s : h->udvst) r |= mk_udv(s);
  r |= dalloc(h, &h->TP, B * NN); r |= dalloc(h, &h->Qb, B * NN); r |= dalloc(h, &h->RHS, B * NN);
  r |= dalloc(h, &h->QRw, B * NN); r |= dalloc(h, &h->qkeys, B * N);
  h->gws_elems = 4ll * B * NN;
  r |= dalloc(h, &h->gws, (size_t)h->gws_elems);
  h->ltau = d.ltau;
  if (h->ltau) {
    const size_t N2 = 2 * N, NN2 = N2 * N2;
    r |= dalloc(h, &h->GT0, B * NN); r |= dalloc(h, &h->G0T, B * NN); r |= dalloc(h, &h->G00, B * NN);
    r |= dalloc(h, &h->GTT, B * NN);
    for (int k = 0; k < 4; ++k) r |= dalloc(h, &h->Hn[k], B * NN);
    r |= dalloc(h, &h->udvr_tau.U, B * NN); r |= dalloc(h, &h->udvr_tau.V, B * NN);
    r |= dalloc(h, &h->udvr_tau.D, B * N); r |= dalloc(h, &h->udvr_tau.detU, B);
    r |= dalloc(h, &h->HB1, B * NN2); r |= dalloc(h, &h->HB2, B * NN2); r |= dalloc(h, &h->HLP, B * NN2);
    r |= dalloc(h, &h->tau2, B * N2); r |= dalloc(h, &h->jpvt2, B * N2); r |= dalloc(h, &h->D3, B * N2);
    r |= dalloc(h, &h->vn2, B * 2 * N2); r |= dalloc(h, &h->info2, B); r |= dalloc(h, &h->first2, B);
    r |= dalloc(h, &h->cmp_tau, 8 * B); r |= dalloc(h, &h->V1I, B * NN); r |= dalloc(h, &h->Qt, B * NN);
    r |= dalloc(h, &h->Gq, 4 * B * NN);
  }
  if (h->df_qr) r |= dalloc(h, &h->QRdf, B * NN);
  if (h->qrr_ok == 2) r |= dalloc(h, &h->qrr_ws, B * qrr_rows_elems(h->N, h->CLr));
  if (h->qr2_mode == 2) r |= dalloc(h, &h->qr2_ws, B * qrr_rows_elems(2 * h->N, h->CL2));
  r |= dalloc(h, &h->Vtmp, B * NN);
  r |= dalloc(h, &h->tau, B * N); r |= dalloc(h, &h->jpvt, B * N); r |= dalloc(h, &h->perm, B * N);
  r |= dalloc(h, &h->iperm, B * N); r |= dalloc(h, &h->DUP, B * N); r |= dalloc(h, &h->vn, B * 2 * N);
  r |= dalloc(h, &h->info, B); r |= dalloc(h, &h->dphase, B); r |= dalloc(h, &h->cmp, 2 * B);
  r |= dalloc(h, &h->opang, B);
  r |= dalloc(h, &h->m, 2 * (C + B)); r |= dalloc(h, &h->sites, C * UPD_KMAX);  // m: one set per block parity
  r |= dalloc(h, &h->Gsnap, B * UPD_KMAX * UPD_KMAX); r |= dalloc(h, &h->Gsub, B * UPD_KMAX * UPD_KMAX);
  r |= dalloc(h, &h->posn, C * UPD_KMAX); r |= dalloc(h, &h->npos, C);
  r |= dalloc(h, &h->W, C * 2 * UPD_KMAX * UPD_KMAX); r |= dalloc(h, &h->dlt, C * 2 * UPD_KMAX);
  r |= dalloc(h, &h->X, C * 2 * N * UPD_KMAX); r |= dalloc(h, &h->Y, C * 2 * N * UPD_KMAX);
  r |= dalloc(h, &h->phase, C); r |= dalloc(h, &h->cnt, 4 * C); r |= dalloc(h, &h->stat, 8 * C);
  r |= dalloc(h, &h->err, 1);
  r |= dalloc(h, &h->draws, C * 6 * M * L);
  r |= dalloc(h, &h->rngkey, C); r |= dalloc(h, &h->rngctr, C);
  if (r) return fail(ALFGPU_ERROR_CUDA);
  if (h->mixed && !(d.reserved[0] & ALFGPU_FLAG_NO_TENSOR_GEMM)) {
    const int e = oz_setup(h);
    if (e) return fail(e);
    h->oz_stab = h->oz && !(d.reserved[0] & ALFGPU_FLAG_FP64_STAB_GEMM) && !h->df_stab;
  }
  h->h_key.assign(C, 0); h->h_ctr.assign(C, 0);
  for (size_t c = 0; c < C; ++c) { h->h_key[c] = alf_chain_key(0, c); h->h_ctr[c] = M * L; }
  *out = h;
  return ALFGPU_ERROR_NONE;
}

void alfgpu_destroy(alfgpu_t* h) {
  if (!h) return;
  cudaSetDevice(h->dev);
  if (h->st) cudaStreamSynchronize(h->st);
  drop_graphs(h);
  for (void* p : h->allocs) cudaFree(p);
  if (h->obs_host) cudaFreeHost(h->obs_host);
  if (h->tau_host) cudaFreeHost(h->tau_host);
  if (h->phase_host) cudaFreeHost(h->phase_host);
  for (cudaEvent_t e : h->ev_pool) cudaEventDestroy(e);
  if (h->ev_fork) cudaEventDestroy(h->ev_fork);
  if (h->ev_join) cudaEventDestroy(h->ev_join);
  if (h->st2) cudaStreamDestroy(h->st2);
  if (h->st) cudaStreamDestroy(h->st);
  delete h;
}

void* alfgpu_stream(alfgpu_t* h) { return h ? (void*)h->st : nullptr; }

int alfgpu_set_profiling(alfgpu_t* h, int32_t enable) {
  if (!h) return ALFGPU_ERROR_ARGUMENT;
  prof_collect(h);
  h->profiling = enable ? 1 : 0;
  for (int i = 0; i < ALFGPU_PROF_N; ++i) { h->prof_ms[i] = 0.0; h->prof_n[i] = 0; }
  return 0;
}

int64_t alfgpu_launch_count(alfgpu_t* h) { return h ? (int64_t)h->launches : -1; }

int alfgpu_get_profile(alfgpu_t* h, double* ms, int64_t* launches) {
  if (!h || !ms || !launches) return ALFGPU_ERROR_ARGUMENT;
  prof_collect(h);
  for (int i = 0; i < ALFGPU_PROF_N; ++i) { ms[i] = h->prof_ms[i]; launches[i] = h->prof_n[i]; }
  return 0;
}

// Rotated basis for two-site vertices with one shared eigenbasis on disjoint site pairs
// (Kondo's J_K vertices): with W = I except the 2x2 block U on every pair, each vertex
// exponential U diag(exp(g phi E)) U^H is diagonal in x' = W^H x.  Op_Wrapup / Op_Wrapdo
// with N_type 1 and 2 (Operator_mod.F90:743-951) rotate into and out of this basis
// around every update; the library stays in it for the whole sweep: expT' = W^H expT W,
// G' = W^H G W, and every G handed out is rotated back.
static void rotate_host(const alfgpu_s* h, double* X, int N) {
  // X <- W^T X W for the real orthogonal W (pairs and U of the handle)
  const double* U = h->rot_U;
  for (const auto& pr : h->rot_pairs) {
    const int a = pr.first, b = pr.second;
    for (int j = 0; j < N; ++j) {  // rows: W^T X
      const double xa = X[a + (size_t)j * N], xb = X[b + (size_t)j * N];
      X[a + (size_t)j * N] = U[0] * xa + U[1] * xb;  // U^T(0,:) = (U00, U10)
      X[b + (size_t)j * N] = U[2] * xa + U[3] * xb;  // U^T(1,:) = (U01, U11)
    }
    for (int i = 0; i < N; ++i) {  // columns: X W
      const double xa = X[i + (size_t)a * N], xb = X[i + (size_t)b * N];
      X[i + (size_t)a * N] = xa * U[0] + xb * U[1];
      X[i + (size_t)b * N] = xa * U[2] + xb * U[3];
    }
  }
}

static int upload_expT(alfgpu_t* h) {
  const size_t NN = (size_t)h->N * h->N;
  std::vector<double> a(h->h_expT), b(h->h_expTinv);
  if (h->rot)
    for (int f = 0; f < h->F; ++f) {
      rotate_host(h, a.data() + f * NN, h->N);
      rotate_host(h, b.data() + f * NN, h->N);
    }
  CK(cudaMemcpy(h->expT, a.data(), h->F * NN * sizeof(double), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(h->expTinv, b.data(), h->F * NN * sizeof(double), cudaMemcpyHostToDevice));
  RET(oz_slice_expT(h));
  CK(cudaStreamSynchronize(h->st));
  return 0;
}

int alfgpu_upload_hopping(alfgpu_t* h, const double* expT, const double* expTinv) {
  if (!h || !expT || !expTinv) return ALFGPU_ERROR_ARGUMENT;
  const size_t NN = (size_t)h->N * h->N;
  for (size_t i = 0; i < h->F * NN; ++i)
    if (!std::isfinite(expT[i]) || !std::isfinite(expTinv[i])) return ALFGPU_ERROR_HAMILTONIAN;
  h->h_expT.assign(expT, expT + h->F * NN);
  h->h_expTinv.assign(expTinv, expTinv + h->F * NN);
  RET(upload_expT(h));
  h->hop_ok = true;
  return 0;
}

// Delayed-update blocks of both passes: consecutive visits with at most kblk positions
// (one per non-zero eigenvalue) on distinct sites.
static int make_blocks(alfgpu_s* h) {
  const int M = h->M, N = h->N;
  for (int dir = 0; dir < 2; ++dir) {
    std::vector<int>& st = h->blk_start[dir];
    std::vector<int>& nc = h->blk_cnt[dir];
    std::vector<int>& pe = h->blk_phase_end[dir];
    st.clear(); nc.clear(); pe.clear();
    std::vector<int> seen(N, 0);
    int npos = 0, prev_ph = -1;
    for (int pos = 0; pos < M; ++pos) {
      const int n = dir == 0 ? pos : M - 1 - pos;
      const int s1 = h->hv_site[n], s2 = h->hv_blk2[n], w = h->hv_nsite[n];
      if (s2 == s1) return ALFGPU_ERROR_UNSUPPORTED;
      const bool clash = seen[s1] || (s2 >= 0 && seen[s2]);
      const int ph = h->pairblock ? h->ph_of[n] : 0;
      if (st.empty() || npos + w > h->kblk || clash || ph != prev_ph) {
        if (!st.empty() && ph != prev_ph) pe.back() = prev_ph;  // the previous block closes its phase
        st.push_back(pos); nc.push_back(0); pe.push_back(-1);
        std::fill(seen.begin(), seen.end(), 0);
        npos = 0;
      }
      prev_ph = ph;
      seen[s1] = 1;
      if (s2 >= 0) seen[s2] = 1;
      npos += w;
      nc.back()++;
    }
    if (!pe.empty()) pe.back() = prev_ph;
  }
  return 0;
}

int alfgpu_upload_vertices(alfgpu_t* h, int32_t chain, const alfgpu_vertices* v) {
  if (!h || !v || chain < -1 || chain >= h->C) return ALFGPU_ERROR_ARGUMENT;
  const int F = h->F, M = h->M, N = h->N;
  const size_t K = (size_t)F * M;
  std::vector<int> site(K), site2(K, -1);
  std::vector<int8_t> nsite(K);
  std::vector<zd> g(K), al(K), ee(K * 10);
  std::vector<double> E(2 * K);
  std::vector<int8_t> ty(K);
  std::vector<std::pair<int, int>> pairs;
  double U[4] = {1.0, 0.0, 0.0, 1.0};
  bool have_rot = false;
  for (size_t k = 0; k < K; ++k) {
    const int n = v->op_n[k], nz = v->op_nz[k];
    if (n < 1 || n > 2 || nz < 1 || nz > n) return ALFGPU_ERROR_UNSUPPORTED;
    if (v->op_type[k] != 1 && v->op_type[k] != 2) return ALFGPU_ERROR_UNSUPPORTED;
    for (int a = 0; a < n; ++a)
      if (v->op_P[2 * k + a] < 0 || v->op_P[2 * k + a] >= N) return ALFGPU_ERROR_HAMILTONIAN;
    if (!v->op_diag[k]) {  // non-diagonal: two sites, real eigenbasis shared by all such vertices
      if (n != 2) return ALFGPU_ERROR_UNSUPPORTED;
      double u[4];
      for (int e = 0; e < 4; ++e) {
        u[e] = v->op_U[(4 * k + e) * 2];
        if (std::fabs(v->op_U[(4 * k + e) * 2 + 1]) > 1e-14) return ALFGPU_ERROR_UNSUPPORTED;
      }
      if (!have_rot) { memcpy(U, u, sizeof(U)); have_rot = true; }
      for (int e = 0; e < 4; ++e)
        if (std::fabs(u[e] - U[e]) > 1e-13) return ALFGPU_ERROR_UNSUPPORTED;
      if (k < (size_t)M) pairs.emplace_back(v->op_P[2 * k], v->op_P[2 * k + 1]);
    }
    nsite[k] = (int8_t)nz;
    site[k] = v->op_P[2 * k];
    if (nz == 2) site2[k] = v->op_P[2 * k + 1];
    g[k] = zmk(v->op_g[2 * k], v->op_g[2 * k + 1]);
    al[k] = zmk(v->op_alpha[2 * k], v->op_alpha[2 * k + 1]);
    E[2 * k] = v->op_E[2 * k];
    E[2 * k + 1] = v->op_E[2 * k + 1];
    ty[k] = (int8_t)v->op_type[k];
    for (int m = 0; m < 2; ++m)
      for (int s = 0; s < 5; ++s)
        ee[k * 10 + m * 5 + s] = zmk(v->op_Eexp[(k * 10 + m * 5 + s) * 2], v->op_Eexp[(k * 10 + m * 5 + s) * 2 + 1]);
    for (int s = 0; s < 10; ++s)
      if (ee[k * 10 + s].y != 0.0) h->eexp_complex = 1;
    if (!std::isfinite(g[k].x) || !std::isfinite(g[k].y)) return ALFGPU_ERROR_HAMILTONIAN;
  }
  // the vertices of every flavour act on the same sites
  for (int n = 0; n < M; ++n)
    for (int f = 1; f < F; ++f) {
      const size_t k = (size_t)f * M + n;
      if (site[k] != site[n] || site2[k] != site2[n] || v->op_diag[k] != v->op_diag[n]) return ALFGPU_ERROR_UNSUPPORTED;
    }
  // Kinds: 0 one position, 1 two diagonal positions (a non-diagonal vertex in the rotated basis
  // or a diagonal two-site one), 2 vector (a single-site vertex on a site of a rotated pair: in
  // the rotated basis e_a becomes u = W^T e_a on the pair).  Rotated pairs are disjoint, each of
  // their sites belongs to exactly one non-diagonal vertex, and other vertices touch them only
  // as single-site (vector) vertices.
  std::vector<int8_t> kind(K, 0);
  std::vector<int> blk2(K, -1);
  std::vector<double> vc(2 * K, 0.0);
  for (size_t k = 0; k < K; ++k)
    if (nsite[k] == 2) { kind[k] = 1; blk2[k] = site2[k]; }
  int pairblock = 0;
  std::vector<int> ph_of, ph_n0, ph_n1;
  if (have_rot) {
    std::vector<int> partner(N, -1), slot(N, -1), cnt_nd(N, 0);
    for (const auto& pr : pairs) {
      partner[pr.first] = pr.second; partner[pr.second] = pr.first;
      slot[pr.first] = 0; slot[pr.second] = 1;
    }
    for (int n = 0; n < M; ++n)
      if (!v->op_diag[n]) { cnt_nd[site[n]]++; cnt_nd[v->op_P[2 * n + 1]]++; }
    for (int i = 0; i < N; ++i)
      if (partner[i] >= 0 && cnt_nd[i] != 1) return ALFGPU_ERROR_UNSUPPORTED;
    for (size_t k = 0; k < K; ++k) {
      if (!v->op_diag[k]) continue;
      const int a = v->op_P[2 * k];
      if (v->op_n[k] == 2) {
        if (partner[a] >= 0 || partner[v->op_P[2 * k + 1]] >= 0) return ALFGPU_ERROR_UNSUPPORTED;
        continue;
      }
      if (partner[a] < 0) continue;
      kind[k] = 2;
      blk2[k] = partner[a];
      vc[2 * k] = slot[a] == 0 ? U[0] : U[3];      // coefficient on a
      vc[2 * k + 1] = slot[a] == 0 ? U[2] : U[1];  // coefficient on its partner
      pairblock = 1;
    }
    if (chain >= 0 && (!h->rot || h->rot_pairs != pairs)) {
      if (h->vert_ok) return ALFGPU_ERROR_UNSUPPORTED;  // per-chain tables share one basis
    }
  }
  if (pairblock) {  // phases: a vertex whose support meets the current phase's opens the next one
    std::vector<int> mark(N, -1);
    int cur = 0;
    ph_of.assign(M, 0);
    ph_n0.push_back(0);
    for (int n = 0; n < M; ++n) {
      const int a = site[n], b = blk2[n];
      if (mark[a] == cur || (b >= 0 && mark[b] == cur)) { ph_n1.push_back(n); ph_n0.push_back(n); ++cur; }
      mark[a] = cur;
      if (b >= 0) mark[b] = cur;
      ph_of[n] = cur;
    }
    ph_n1.push_back(M);
  }
  if (chain >= 0 && h->vert_ok && (pairblock != h->pairblock || ph_n0 != h->ph_n0))
    return ALFGPU_ERROR_UNSUPPORTED;  // the chains of a handle share one phase structure
  h->pairblock = pairblock;
  h->ph_of = ph_of; h->ph_n0 = ph_n0; h->ph_n1 = ph_n1;
  h->hv_site.assign(site.begin(), site.begin() + M);
  h->hv_site2.assign(site2.begin(), site2.begin() + M);
  h->hv_nsite.assign(nsite.begin(), nsite.begin() + M);
  h->hv_blk2.assign(blk2.begin(), blk2.begin() + M);
  RET(make_blocks(h));
  // transition factors for every (vertex, old field, flip choice); type-1 fields flip sign
  std::vector<UpdTab> tab(K * 15);
  for (size_t k = 0; k < K; ++k) {
    const int t = ty[k] - 1;
    for (int so = -2; so <= 2; ++so)
      for (int ch = 0; ch < 3; ++ch) {
        const int sn = (t == 0) ? -so : h->ft.flip[so + 2][ch];
        UpdTab& e = tab[(k * 5 + so + 2) * 3 + ch];
        if (sn < -2 || sn > 2) {
          for (int m = 0; m < 2; ++m) { e.myexp[m] = zmk(1.0, 0.0); e.dlt[m] = zmk(0.0, 0.0); }
          e.expal = zmk(1.0, 0.0);
          continue;
        }
        const double dphi = h->ft.phi[t][sn + 2] - h->ft.phi[t][so + 2];
        const std::complex<double> Z1(g[k].x * dphi, g[k].y * dphi);
        for (int m = 0; m < 2; ++m) {
          const std::complex<double> me = std::exp(Z1 * E[2 * k + m]);
          e.myexp[m] = zmk(me.real(), me.imag());
          e.dlt[m] = zmk(me.real() - 1.0, me.imag());
        }
        const std::complex<double> ea = std::exp(Z1 * std::complex<double>(al[k].x, al[k].y));
        e.expal = zmk(ea.real(), ea.imag());
      }
  }
  // positions of each site, ascending (vertex n, eigen-index I) -> 2n + I, per flavour
  std::vector<int> sptr((size_t)F * (N + 1), 0), slist((size_t)2 * K);
  for (int f = 0; f < F; ++f) {
    int* ptr = &sptr[(size_t)f * (N + 1)];
    for (int n = 0; n < M; ++n) {
      const size_t k = (size_t)f * M + n;
      ptr[site[k] + 1]++;
      if (site2[k] >= 0) ptr[site2[k] + 1]++;
    }
    for (int i = 0; i < N; ++i) ptr[i + 1] += ptr[i];
    std::vector<int> fill(ptr, ptr + N);
    for (int n = 0; n < M; ++n) {
      const size_t k = (size_t)f * M + n;
      slist[(size_t)f * 2 * M + fill[site[k]]++] = 2 * n;
      if (site2[k] >= 0) slist[(size_t)f * 2 * M + fill[site2[k]]++] = 2 * n + 1;
    }
  }
  int c0 = chain < 0 ? 0 : chain, c1 = chain < 0 ? h->C : chain + 1;
  for (int c = c0; c < c1; ++c) {
    CK(cudaMemcpy(h->v_tab + c * K * 15, tab.data(), K * 15 * sizeof(UpdTab), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(h->v_sptr + (size_t)c * F * (N + 1), sptr.data(), sptr.size() * sizeof(int), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(h->v_slist + (size_t)c * 2 * K, slist.data(), 2 * K * sizeof(int), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(h->v_site + c * K, site.data(), K * sizeof(int), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(h->v_site2 + c * K, site2.data(), K * sizeof(int), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(h->v_nsite + c * K, nsite.data(), K, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(h->v_g + c * K, g.data(), K * sizeof(zd), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(h->v_alpha + c * K, al.data(), K * sizeof(zd), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(h->v_type + c * K, ty.data(), K, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(h->v_Eexp + c * K * 10, ee.data(), K * 10 * sizeof(zd), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(h->v_kind + c * K, kind.data(), K, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(h->v_blk2 + c * K, blk2.data(), K * sizeof(int), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(h->v_vc + 2 * c * K, vc.data(), 2 * K * sizeof(double), cudaMemcpyHostToDevice));
  }
  const bool rot_changed = have_rot != h->rot || (have_rot && (pairs != h->rot_pairs || memcmp(U, h->rot_U, sizeof(U))));
  h->rot = have_rot;
  h->rot_pairs = pairs;
  memcpy(h->rot_U, U, sizeof(U));
  if (have_rot) {
    std::vector<int> pp(2 * pairs.size());
    for (size_t i = 0; i < pairs.size(); ++i) { pp[2 * i] = pairs[i].first; pp[2 * i + 1] = pairs[i].second; }
    if (!h->rot_dev) {
      void* q = nullptr;
      CK(cudaMalloc(&q, (size_t)N * sizeof(int)));
      h->allocs.push_back(q);
      h->rot_dev = (int*)q;
    }
    CK(cudaMemcpy(h->rot_dev, pp.data(), pp.size() * sizeof(int), cudaMemcpyHostToDevice));
  }
  if (rot_changed && h->hop_ok) RET(upload_expT(h));
  drop_graphs(h);  // block partition and basis may have changed
  h->vert_ok = true;
  return 0;
}

int alfgpu_set_fields(alfgpu_t* h, int32_t chain, const int8_t* f) {
  if (!h || !f || chain < 0 || chain >= h->C) return ALFGPU_ERROR_ARGUMENT;
  const size_t ML = (size_t)h->M * h->L;
  for (size_t i = 0; i < ML; ++i)
    if (f[i] != 1 && f[i] != -1 && f[i] != 2 && f[i] != -2) return ALFGPU_ERROR_FIELDS;
  CK(cudaMemcpy(h->fields + chain * ML, f, ML, cudaMemcpyHostToDevice));
  h->fields_ok = true;
  return 0;
}

int alfgpu_set_fields_c128(alfgpu_t* h, int32_t chain, const double* f) {
  if (!h || !f) return ALFGPU_ERROR_ARGUMENT;
  const size_t ML = (size_t)h->M * h->L;
  std::vector<int8_t> b(ML);
  for (size_t i = 0; i < ML; ++i) {
    const double x = f[2 * i];  // nsigma%f stores the discrete field values as complex numbers
    if (!(x == 1.0 || x == -1.0 || x == 2.0 || x == -2.0) || f[2 * i + 1] != 0.0) return ALFGPU_ERROR_FIELDS;
    b[i] = (int8_t)x;
  }
  return alfgpu_set_fields(h, chain, b.data());
}

int alfgpu_get_fields(alfgpu_t* h, int32_t chain, int8_t* f) {
  if (!h || !f || chain < 0 || chain >= h->C) return ALFGPU_ERROR_ARGUMENT;
  const size_t ML = (size_t)h->M * h->L;
  CK(cudaStreamSynchronize(h->st));
  CK(cudaMemcpy(f, h->fields + chain * ML, ML, cudaMemcpyDeviceToHost));
  return 0;
}

int alfgpu_get_rng_state(alfgpu_t* h, int32_t chain, uint64_t* key, uint64_t* counter) {
  if (!h || chain < 0 || chain >= h->C || !key || !counter) return ALFGPU_ERROR_ARGUMENT;
  *key = h->h_key[chain];
  *counter = h->h_ctr[chain];
  return 0;
}

int alfgpu_set_rng_state(alfgpu_t* h, int32_t chain, uint64_t key, uint64_t counter) {
  if (!h || chain < 0 || chain >= h->C) return ALFGPU_ERROR_ARGUMENT;
  h->h_key[chain] = key;
  h->h_ctr[chain] = counter;
  return 0;
}

int alfgpu_set_rng(alfgpu_t* h, int32_t chain, uint64_t seed, uint64_t counter) {
  if (!h || chain < 0 || chain >= h->C) return ALFGPU_ERROR_ARGUMENT;
  h->h_key[chain] = alf_chain_key(seed, (uint64_t)chain);
  h->h_ctr[chain] = counter;
  return 0;
}

static int check_err(alfgpu_s* h) {
  int e = 0;
  CK(cudaStreamSynchronize(h->st));
  CK(cudaMemcpy(&e, h->err, sizeof(int), cudaMemcpyDeviceToHost));
  if (e) {
    CK(cudaMemset(h->err, 0, sizeof(int)));
    if (e & 1) return ALFGPU_ERROR_NAN;
    if (e & 2) return ALFGPU_ERROR_UNSTABLE_MATRIX;
    if (e & 4) return ALFGPU_ERROR_TIMEOUT;
    return ALFGPU_ERROR_GENERIC;
  }
  return 0;
}

int alfgpu_init_state(alfgpu_t* h, double* phase_out) {
  if (!h) return ALFGPU_ERROR_ARGUMENT;
  if (!h->hop_ok || !h->vert_ok || !h->fields_ok) return ALFGPU_ERROR_ARGUMENT;
  CK(cudaSetDevice(h->dev));
  RET(udv_reset(h, h->udvl));
  RET(udv_reset(h, h->udvr));
  RET(udv_reset(h, h->udvst[h->Nstm - 1]));
  for (int nst = h->Nstm - 1; nst >= 1; --nst) {
    RET(wrapul(h, h->stab_nt[nst + 1], h->stab_nt[nst]));
    RET(udv_copy(h, h->udvst[nst - 1], h->udvl));
  }
  RET(wrapul(h, h->stab_nt[1], 0));
  RET(stabilise(h, 1, 0));
  RET(check_err(h));
  if (phase_out) CK(cudaMemcpy(phase_out, h->phase, h->C * sizeof(zd), cudaMemcpyDeviceToHost));
  h->state_ok = true;
  return 0;
}

// The sweep proper (main.F90:714-887): everything between the host copies of the draws and
// the error check, so that it can be captured once into a CUDA graph and replayed.
static int sweep_body(alfgpu_s* h, const double* dr, alfgpu_obs_cb cb, void* ctx) {
  const int L = h->L, M = h->M, Nstm = h->Nstm;
  h->rec_stab = 0;
  // up pass (main.F90:717-774)
  RET(udv_reset(h, h->udvr));
  int NST = 1;
  int pending = 0;
  const int pb = h->pairblock;  // vector vertices: every phase's wraps are explicit, none deferred
  for (int ntau = 0; ntau < L; ++ntau) {
    const int ntau1 = ntau + 1;
    RET(hop(h, 1, pending));
    if (pb) {  // the slice's fields before their update, for the explicit phase wraps
      k_copy_fields<<<dim3((M + 255) / 256, h->C), 256, 0, h->st>>>(h->fields, L, M, ntau1, h->fields_old);
      CKL();
    } else {
      RET(slice_scale(h, ntau1));  // vertex wraps of this slice use the fields before their update
    }
    RET(update_slice(h, ntau1, 0, ntau * M, dr));
    pending = pb ? 0 : 1;
    if (ntau1 == h->stab_nt[NST]) {
      if (pending) {
        dim3 grid((unsigned)(((long long)h->N * h->N + 255) / 256), h->B);
        k_apply_scale<<<grid, 256, 0, h->st>>>(h->G, h->S, h->Sinv, h->N);
        CKL();
      }
      pending = 0;
      RET(wrapur(h, h->stab_nt[NST - 1], ntau1));
      RET(udv_copy(h, h->udvl, h->udvst[NST - 1]));
      RET(udv_copy(h, h->udvst[NST - 1], h->udvr));
      const int nvar = (ntau1 > L / 2) ? 2 : 1;
      RET(stabilise(h, nvar, 1));
      NST++;
    }
    RET(obs_eq(h, cb, ctx, ntau1, pending));  // LOBS_ST = 1, LOBS_EN = Ltrot
  }
  // down pass (main.F90:776-834)
  RET(udv_reset(h, h->udvl));
  NST = Nstm - 1;
  for (int ntau = L; ntau >= 1; --ntau) {
    const int ntau1 = ntau - 1;
    RET(update_slice(h, ntau, 1, L * M + (L - ntau) * M, dr));
    if (!pb) RET(slice_scale(h, ntau));  // Op_Wrapdo N_type=1 uses the updated fields
    RET(hop(h, 0, pb ? 0 : 1));
    if (ntau1 >= 1) RET(obs_eq(h, cb, ctx, ntau1, 0));
    if (NST >= 1 && h->stab_nt[NST] == ntau1 && ntau1 != 0) {
      RET(wrapul(h, h->stab_nt[NST + 1], ntau1));
      RET(udv_copy(h, h->udvr, h->udvst[NST - 1]));
      RET(udv_copy(h, h->udvst[NST - 1], h->udvl));
      const int nvar = (ntau1 > L / 2) ? 2 : 1;
      RET(stabilise(h, nvar, 1));
      NST--;
    }
  }
  // G on time slice 0 (main.F90:836-872)
  RET(wrapul(h, h->stab_nt[1], h->stab_nt[0]));
  RET(udv_reset(h, h->udvr));
  RET(stabilise(h, 1, 1));
  RET(udv_reset(h, h->udvst[Nstm - 1]));
  if (h->ltau) RET(tau_m(h, cb, ctx));  // main.F90:879-881
  k_count_sweep<<<(h->C + 127) / 128, 128, 0, h->st>>>(h->stat, h->C);
  CKL();
  return 0;
}

// The launch part of alfgpu_sweep: everything up to the last launch of the sweep on h->st (graph
// replay when it applies), without waiting for the GPU.
static int sweep_launch(alfgpu_t* h, const double* uniforms, alfgpu_obs_cb cb, void* ctx) {
  if (!h) return ALFGPU_ERROR_ARGUMENT;
  if (!h->state_ok) return ALFGPU_ERROR_ARGUMENT;
  CK(cudaSetDevice(h->dev));
  const int L = h->L, M = h->M;
  const double* dr = nullptr;
  if (uniforms) {
    CK(cudaMemcpyAsync(h->draws, uniforms, (size_t)h->C * 6 * M * L * sizeof(double), cudaMemcpyHostToDevice, h->st));
    dr = h->draws;
  } else {
    CK(cudaMemcpyAsync(h->rngkey, h->h_key.data(), h->C * sizeof(unsigned long long), cudaMemcpyHostToDevice, h->st));
    CK(cudaMemcpyAsync(h->rngctr, h->h_ctr.data(), h->C * sizeof(unsigned long long), cudaMemcpyHostToDevice, h->st));
  }
  // the launch sequence is fixed for a handle, so the sweep is captured once into a graph
  // (per draw source) and replayed; callbacks, recording, profiling and TAU_M's buffer
  // rotation run the stream path
  const int gi = uniforms ? 1 : 0;
  if (h->use_graph && !cb && !h->profiling && !h->recording && !h->ltau) {
    if (!h->gexec[gi]) {
      const long long l0 = h->launches;
      CK(cudaStreamBeginCapture(h->st, cudaStreamCaptureModeThreadLocal));
      const int rc = sweep_body(h, dr, nullptr, nullptr);
      cudaGraph_t graph = nullptr;
      const cudaError_t ce = cudaStreamEndCapture(h->st, &graph);
      if (rc || ce != cudaSuccess) {
        if (graph) cudaGraphDestroy(graph);
        h->launches = l0;
        if (rc) return rc;
        h->last_cuda = ce;
        h->last_line = __LINE__;
        return ALFGPU_ERROR_CUDA;
      }
      const cudaError_t ie = cudaGraphInstantiate(&h->gexec[gi], graph, 0);
      cudaGraphDestroy(graph);
      if (ie != cudaSuccess) {
        h->gexec[gi] = nullptr;
        h->last_cuda = ie;
        h->last_line = __LINE__;
        return ALFGPU_ERROR_CUDA;
      }
      h->glaunches[gi] = h->launches - l0;
      h->launches = l0;
    }
    CK(cudaGraphLaunch(h->gexec[gi], h->st));
    h->launches += h->glaunches[gi];
  } else {
    RET(sweep_body(h, dr, cb, ctx));
  }
  if (!uniforms)
    for (int c = 0; c < h->C; ++c) h->h_ctr[c] += 6ull * M * L;
  return 0;
}

// The end of a sweep: wait for h->st, read the device error flags, collect the phase profile.
static int sweep_finish(alfgpu_t* h) {
  CK(cudaSetDevice(h->dev));
  const int rc = check_err(h);
  prof_collect(h);
  return rc;
}

int alfgpu_sweep(alfgpu_t* h, const double* uniforms, alfgpu_obs_cb cb, void* ctx) {
  RET(sweep_launch(h, uniforms, cb, ctx));
  return sweep_finish(h);
}

int alfgpu_sweep_many(alfgpu_t* const* hs, int32_t n, const double* const* uniforms, int32_t* status) {
  if (!hs || n < 0 || !status) return ALFGPU_ERROR_ARGUMENT;
  for (int k = 0; k < n; ++k)
    if (!hs[k]) return ALFGPU_ERROR_ARGUMENT;
  int first = 0;
  std::vector<char> launched(n, 0);
  for (int k = 0; k < n; ++k) {  // every handle's launches first: they run on their own streams
    status[k] = sweep_launch(hs[k], uniforms ? uniforms[k] : nullptr, nullptr, nullptr);
    launched[k] = status[k] == 0;
  }
  for (int k = 0; k < n; ++k) {
    if (launched[k]) status[k] = sweep_finish(hs[k]);
    if (status[k] && !first) first = status[k];
  }
  return first;
}


int alfgpu_set_delay(alfgpu_t* h, int32_t k) {
  if (!h || k < 2 || k > UPD_KMAX) return ALFGPU_ERROR_ARGUMENT;
  h->kblk = k;
  if (h->vert_ok) RET(make_blocks(h));
  drop_graphs(h);
  return 0;
}

// Stabilisation interval (control of the stabilisation drift): re-plans the stabilisation
// points (Stab_nt of main.F90:446-457 with the new Nwrap) and grows the UDV stack as needed.
// G and the stack belong to the old points afterwards, so alfgpu_init_state must run before
// the next sweep.
int alfgpu_set_nwrap(alfgpu_t* h, int32_t nwrap) {
  if (!h || nwrap < 1 || nwrap > h->L) return ALFGPU_ERROR_ARGUMENT;
  CK(cudaSetDevice(h->dev));
  CK(cudaStreamSynchronize(h->st));
  const int L = h->L;
  const int nstm = (L % nwrap == 0) ? L / nwrap : L / nwrap + 1;
  const size_t N = h->N, NN = N * N, B = h->B;
  while ((int)h->udvst.size() < nstm) {
    UDVSet s;
    int q = 0;
    q |= dalloc(h, &s.U, B * NN); q |= dalloc(h, &s.V, B * NN); q |= dalloc(h, &s.D, B * N); q |= dalloc(h, &s.detU, B);
    if (q) return ALFGPU_ERROR_CUDA;
    h->udvst.push_back(s);
  }
  if (h->rec_acc && nstm > h->rec_nstm) {
    const size_t P = 2 * (size_t)nstm;
    int r = 0;
    r |= dalloc(h, &h->rec_G, P * B * NN);
    r |= dalloc(h, &h->rec_Gw, P * B * NN);
    r |= dalloc(h, &h->rec_phase, P * h->C);
    if (r) return ALFGPU_ERROR_CUDA;
    h->rec_nstm = nstm;
  }
  h->Nstm = nstm;
  h->d.nwrap = nwrap;
  h->stab_nt.assign(nstm + 1, 0);
  for (int n = 1; n < nstm; ++n) h->stab_nt[n] = nwrap * n;
  h->stab_nt[nstm] = L;
  drop_graphs(h);
  h->state_ok = false;
  return 0;
}

int alfgpu_get_nwrap(alfgpu_t* h, int32_t* nwrap) {
  if (!h || !nwrap) return ALFGPU_ERROR_ARGUMENT;
  *nwrap = h->d.nwrap;
  return 0;
}

int alfgpu_get_delay(alfgpu_t* h, int32_t* k) {
  if (!h || !k) return ALFGPU_ERROR_ARGUMENT;
  *k = h->kblk;
  return 0;
}

int alfgpu_tune_delay(alfgpu_t* h, int32_t nsweeps, int32_t* k_out) {
  if (!h || nsweeps < 1) return ALFGPU_ERROR_ARGUMENT;
  if (!h->state_ok || !h->vert_ok) return ALFGPU_ERROR_ARGUMENT;
  const int cand[4] = {8, 16, 24, 32};
  const int prof0 = h->profiling;
  double best = 1e300;
  int kbest = h->kblk;
  for (int c = 0; c < 4; ++c) {
    RET(alfgpu_set_delay(h, cand[c]));
    h->profiling = 1;
    for (int i = 0; i < ALFGPU_PROF_N; ++i) { h->prof_ms[i] = 0.0; h->prof_n[i] = 0; }
    for (int s = 0; s < nsweeps; ++s) RET(alfgpu_sweep(h, nullptr, nullptr, nullptr));
    const double t = h->prof_ms[ALFGPU_PROF_UPDATE] + h->prof_ms[ALFGPU_PROF_FLUSH];
    if (t < best) { best = t; kbest = cand[c]; }
  }
  h->profiling = prof0;
  for (int i = 0; i < ALFGPU_PROF_N; ++i) { h->prof_ms[i] = 0.0; h->prof_n[i] = 0; }
  RET(alfgpu_set_delay(h, kbest));
  if (k_out) *k_out = kbest;
  return 0;
}

int alfgpu_get_green(alfgpu_t* h, int32_t chain, double* G) {
  if (!h || !G || chain < 0 || chain >= h->C) return ALFGPU_ERROR_ARGUMENT;
  const size_t n = (size_t)h->F * h->N * h->N;
  const zd* src = h->G + chain * n;
  if (h->rot) {
    RET(copy_mats(h, h->T1, src, n));
    RET(rotate_out(h, h->T1, h->F));
    src = h->T1;
  }
  CK(cudaStreamSynchronize(h->st));
  CK(cudaMemcpy(G, src, n * sizeof(zd), cudaMemcpyDeviceToHost));
  return 0;
}

int alfgpu_get_phase(alfgpu_t* h, double* phase) {
  if (!h || !phase) return ALFGPU_ERROR_ARGUMENT;
  CK(cudaStreamSynchronize(h->st));
  CK(cudaMemcpy(phase, h->phase, h->C * sizeof(zd), cudaMemcpyDeviceToHost));
  return 0;
}

int alfgpu_get_stats(alfgpu_t* h, int32_t chain, alfgpu_stats* s) {
  if (!h || !s || chain < 0 || chain >= h->C) return ALFGPU_ERROR_ARGUMENT;
  long long cn[4];
  double st[8];
  CK(cudaStreamSynchronize(h->st));
  CK(cudaMemcpy(cn, h->cnt + 4 * chain, sizeof(cn), cudaMemcpyDeviceToHost));
  CK(cudaMemcpy(st, h->stat + 8 * chain, sizeof(st), cudaMemcpyDeviceToHost));
  memset(s, 0, sizeof(*s));
  s->n_prop = cn[0]; s->n_acc = cn[1]; s->n_prop_eff = cn[2]; s->n_acc_eff = cn[3];
  s->ncg = (int64_t)st[0]; s->xmeanG_sum = st[1]; s->xmaxG = st[2]; s->xmaxP = st[3];
  s->ncg_tau = (int64_t)st[4]; s->xmean_tau_sum = st[5]; s->xmax_tau = st[6]; s->sweeps = (int64_t)st[7];
  return 0;
}

int alfgpu_reset_stats(alfgpu_t* h) {
  if (!h) return ALFGPU_ERROR_ARGUMENT;
  CK(cudaMemsetAsync(h->cnt, 0, 4 * h->C * sizeof(long long), h->st));
  CK(cudaMemsetAsync(h->stat, 0, 8 * h->C * sizeof(double), h->st));
  CK(cudaStreamSynchronize(h->st));
  return 0;
}

int alfgpu_set_recording(alfgpu_t* h, int32_t enable) {
  if (!h) return ALFGPU_ERROR_ARGUMENT;
  if (enable && !h->rec_acc) {
    const size_t V = (size_t)2 * h->M * h->L, P = 2 * (size_t)h->Nstm, NN = (size_t)h->N * h->N;
    int r = 0;
    r |= dalloc(h, &h->rec_acc, h->C * V);
    r |= dalloc(h, &h->rec_ratio, h->C * V);
    r |= dalloc(h, &h->rec_G, P * h->B * NN);
    r |= dalloc(h, &h->rec_Gw, P * h->B * NN);
    r |= dalloc(h, &h->rec_phase, P * h->C);
    if (r) return ALFGPU_ERROR_CUDA;
    h->rec_nstm = h->Nstm;
  }
  h->recording = enable ? 1 : 0;
  return 0;
}

int alfgpu_get_record(alfgpu_t* h, int32_t chain, int8_t* acc, double* ratio, double* G_fresh, double* G_wrapped,
                      double* phase) {
  if (!h || chain < 0 || chain >= h->C || !h->rec_acc) return ALFGPU_ERROR_ARGUMENT;
  const size_t V = (size_t)2 * h->M * h->L, P = 2 * (size_t)h->Nstm, NN = (size_t)h->N * h->N, F = h->F;
  CK(cudaStreamSynchronize(h->st));
  if (acc) CK(cudaMemcpy(acc, h->rec_acc + chain * V, V, cudaMemcpyDeviceToHost));
  if (ratio) CK(cudaMemcpy(ratio, h->rec_ratio + chain * V, V * sizeof(zd), cudaMemcpyDeviceToHost));
  for (size_t p = 0; p < P; ++p) {
    const size_t off = (p * h->B + (size_t)chain * F) * NN;
    if (G_fresh) CK(cudaMemcpy(G_fresh + 2 * p * F * NN, h->rec_G + off, F * NN * sizeof(zd), cudaMemcpyDeviceToHost));
    if (G_wrapped)
      CK(cudaMemcpy(G_wrapped + 2 * p * F * NN, h->rec_Gw + off, F * NN * sizeof(zd), cudaMemcpyDeviceToHost));
    if (phase) CK(cudaMemcpy(phase + 2 * p, h->rec_phase + p * h->C + chain, sizeof(zd), cudaMemcpyDeviceToHost));
  }
  return 0;
}

// ---- one-shot component entry points -------------------------------------------------------
static int oneshot_handle(int N, alfgpu_s** out) {
  alfgpu_dims d;
  memset(&d, 0, sizeof(d));
  d.ndim = N; d.n_fl = 1; d.n_sun = 1; d.n_op = 1; d.ltrot = 1; d.nwrap = 1; d.n_chains = 1;
  d.precision = ALFGPU_PRECISION_FP64;
  d.reserved[0] = ALFGPU_FLAG_EXACT_QRP;  // decompose_UDV_state / CGR default branch: ZGEQP3 pivoting
  return alfgpu_create(out, &d);
}

int alfgpu_cgr(int32_t ndim, int32_t nvar, const double* UR, const double* DR, const double* VR, const double* UL,
               const double* DL, const double* VL, double* G, double* phase) {
  if (ndim < 1 || !UR || !DR || !VR || !UL || !DL || !VL || !G || !phase) return ALFGPU_ERROR_ARGUMENT;
  alfgpu_s* h = nullptr;
  RET(oneshot_handle(ndim, &h));
  const size_t N = ndim, NN = N * N;
  auto run = [&]() -> int {
    std::vector<double> dr(N), dl(N);
    for (size_t i = 0; i < N; ++i) { dr[i] = DR[2 * i]; dl[i] = DL[2 * i]; }
    CK(cudaMemcpy(h->udvr.U, UR, NN * sizeof(zd), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(h->udvr.V, VR, NN * sizeof(zd), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(h->udvr.D, dr.data(), N * sizeof(double), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(h->udvl.U, UL, NN * sizeof(zd), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(h->udvl.V, VL, NN * sizeof(zd), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(h->udvl.D, dl.data(), N * sizeof(double), cudaMemcpyHostToDevice));
    // det(U) of arbitrary inputs: pivoted QR of each U (det = det(Q) prod R_ii sign(P))
    for (int side = 0; side < 2; ++side) {
      UDVSet& s = side ? h->udvl : h->udvr;
      RET(qr_any(h, s.U, nullptr, h->QRw, 1));
      QRInfo inf;
      CK(cudaMemcpyAsync(&inf, h->info, sizeof(inf), cudaMemcpyDeviceToHost, h->st));
      CK(cudaStreamSynchronize(h->st));
      std::vector<double> dd(N);
      CK(cudaMemcpy(dd.data(), h->DUP, N * sizeof(double), cudaMemcpyDeviceToHost));
      zd det = zmul(inf.detQ, inf.prodR);
      if (inf.psign < 0) det = zneg(det);
      CK(cudaMemcpy(s.detU, &det, sizeof(zd), cudaMemcpyHostToDevice));
    }
    RET(cgr(h, nvar, h->udvr, h->udvl, h->G));
    CK(cudaMemsetAsync(h->opang, 0, sizeof(double), h->st));
    StabFinishParams sp;
    memset(&sp, 0, sizeof(sp));
    sp.C = 1; sp.F = 1; sp.NSUN = 1; sp.nvar = nvar; sp.compare = 0;
    sp.detUR = h->udvr.detU; sp.detUL = h->udvl.detU; sp.info = h->info; sp.opang = h->opang; sp.cmp = h->cmp;
    sp.phase = h->phase; sp.stat = h->stat; sp.err = h->err;
    k_stab_finish<<<1, 32, 0, h->st>>>(sp);
    CKL();
    CK(cudaStreamSynchronize(h->st));
    CK(cudaMemcpy(G, h->G, NN * sizeof(zd), cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(phase, h->phase, sizeof(zd), cudaMemcpyDeviceToHost));
    return 0;
  };
  int rc = run();
  alfgpu_destroy(h);
  return rc;
}

int alfgpu_decompose(int32_t ndim, char side, double* U, double* D, double* V) {
  if (ndim < 1 || !U || !D || !V) return ALFGPU_ERROR_ARGUMENT;
  const int left = (side == 'l' || side == 'L');
  alfgpu_s* h = nullptr;
  RET(oneshot_handle(ndim, &h));
  const size_t N = ndim, NN = N * N;
  auto run = [&]() -> int {
    std::vector<double> dd(N);
    for (size_t i = 0; i < N; ++i) dd[i] = D[2 * i];
    UDVSet& s = h->udvr;
    CK(cudaMemcpy(s.U, U, NN * sizeof(zd), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(s.V, V, NN * sizeof(zd), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(s.D, dd.data(), N * sizeof(double), cudaMemcpyHostToDevice));
    RET(decompose(h, s, left));
    CK(cudaStreamSynchronize(h->st));
    CK(cudaMemcpy(U, s.U, NN * sizeof(zd), cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(V, s.V, NN * sizeof(zd), cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(dd.data(), s.D, N * sizeof(double), cudaMemcpyDeviceToHost));
    for (size_t i = 0; i < N; ++i) { D[2 * i] = dd[i]; D[2 * i + 1] = 0.0; }
    return 0;
  };
  int rc = run();
  alfgpu_destroy(h);
  return rc;
}

}  // extern "C"

// ---- decompose without device allocation -----------------------------------------------------
// Scratch of alfgpu_decompose_noalloc: a file-scope device array (held by every GPU that loads
// the library, ~1.06 MiB).  Host code must not take the address of g_noalloc_scratch directly:
// in host code the symbol is only a stand-in for the device copy, so each device's address is
// obtained with cudaGetSymbolAddress while that device is current.
struct NoallocScratch {
  zd Vtmp[ALFGPU_NOALLOC_MAX_NDIM * ALFGPU_NOALLOC_MAX_NDIM];
  zd tau[ALFGPU_NOALLOC_MAX_NDIM];
  int jpvt[ALFGPU_NOALLOC_MAX_NDIM];
  int perm[ALFGPU_NOALLOC_MAX_NDIM];
  double DUP[ALFGPU_NOALLOC_MAX_NDIM];
  double vn[2 * ALFGPU_NOALLOC_MAX_NDIM];
  QRInfo info;
  zd dphase;
  zd detU;
};
static __device__ __align__(256) NoallocScratch g_noalloc_scratch;

namespace {
// Per-device set-up of alfgpu_decompose_noalloc.  The first call on a device resolves the
// scratch address under the device's mutex and publishes it with a release store after cl16
// is written, so concurrent first calls from several host threads see either no address (and
// take the mutex) or the address together with cl16.  A failed set-up is retried next call.
struct NoallocDevice {
  std::mutex mu;
  std::atomic<NoallocScratch*> scratch{nullptr};
  int cl16 = 0;  // non-portable 16-CTA clusters enabled for the QR kernels
};
NoallocDevice g_noalloc_dev[64];
}  // namespace

extern "C" int alfgpu_decompose_noalloc(int32_t ndim, char side, double* U, double* D, double* V, double* detU,
                                        void* stream) {
  if (ndim < 1 || !U || !D || !V) return ALFGPU_ERROR_ARGUMENT;
  if (ndim > ALFGPU_NOALLOC_MAX_NDIM) return ALFGPU_ERROR_SIZE;
  if (side != 'r' && side != 'R' && side != 'l' && side != 'L') return ALFGPU_ERROR_ARGUMENT;
  int dev = -1;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return ALFGPU_ERROR_CUDA;
  NoallocDevice& nd = g_noalloc_dev[dev];
  NoallocScratch* s = nd.scratch.load(std::memory_order_acquire);
  if (!s) {  // first call on this device: resolve the device address of the scratch array
    std::lock_guard<std::mutex> lock(nd.mu);
    s = nd.scratch.load(std::memory_order_relaxed);
    if (!s) {
      void* p = nullptr;
      if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) {
        cudaGetLastError();
        return ALFGPU_ERROR_CUDA;
      }
      if (cudaFuncSetAttribute(k_qrp, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) == cudaSuccess &&
          cudaFuncSetAttribute(k_orgqr, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) == cudaSuccess)
        nd.cl16 = 1;
      cudaGetLastError();
      s = static_cast<NoallocScratch*>(p);
      nd.scratch.store(s, std::memory_order_release);
    }
  }
  alfgpu_s ctx;  // host-side bookkeeping only; all device memory below is the caller's or the scratch
  ctx.N = ndim; ctx.F = 1; ctx.C = 1; ctx.B = 1; ctx.M = 1; ctx.L = 1; ctx.NSUN = 1; ctx.dev = dev;
  ctx.CL = cluster_size(ndim);
  if (ctx.CL > 8 && !nd.cl16) ctx.CL = 8;
  ctx.st = (cudaStream_t)stream;
  ctx.Vtmp = s->Vtmp; ctx.tau = s->tau; ctx.jpvt = s->jpvt; ctx.perm = s->perm; ctx.DUP = s->DUP; ctx.vn = s->vn;
  ctx.info = &s->info; ctx.dphase = &s->dphase;
  UDVSet u;
  u.U = reinterpret_cast<zd*>(U);
  u.V = reinterpret_cast<zd*>(V);
  u.D = D;
  u.detU = detU ? reinterpret_cast<zd*>(detU) : &s->detU;
  const int rc = decompose(&ctx, u, (side == 'l' || side == 'L') ? 1 : 0);
  ctx.st = nullptr;  // the caller owns the stream
  return rc;
}

int alfgpu_oz_dgemm(int32_t m, int32_t n, int32_t k, const double* A, int32_t lda, const double* B, int32_t ldb,
                    double* C, int32_t ldc, int32_t device) {
  if (m < 1 || n < 1 || k < 1 || !A || !B || !C || lda < m || ldb < k || ldc < m) return ALFGPU_ERROR_ARGUMENT;
  const int Kp = oz_round(k, OZ_KC);
  int bits = 0, S = 0, bn = 0, nst = 0;
  if (oz_pick(Kp, &bits, &S) || oz_pick_tile(S, Kp / OZ_KC, &bn, &nst)) return ALFGPU_ERROR_SIZE;
  if (!oz_encoder()) return ALFGPU_ERROR_CUDA;
  alfgpu_s* h = new alfgpu_s();
  h->dev = device;
  int rc = 0;
  auto run = [&]() -> int {
    CK(cudaSetDevice(device));
    CK(cudaStreamCreateWithFlags(&h->st, cudaStreamNonBlocking));
    const int RpA = oz_round(m, OZ_BM), RpB = oz_round(n, OZ_BM);
    double *dA = nullptr, *dB = nullptr, *dC = nullptr;
    unsigned short *sa = nullptr, *sb = nullptr;
    int *ea = nullptr, *eb = nullptr;
    int r = 0;
    r |= dalloc(h, &dA, (size_t)m * k); r |= dalloc(h, &dB, (size_t)k * n); r |= dalloc(h, &dC, (size_t)m * n);
    r |= dalloc(h, &sa, (size_t)S * RpA * Kp); r |= dalloc(h, &sb, (size_t)S * RpB * Kp);
    r |= dalloc(h, &ea, (size_t)RpA); r |= dalloc(h, &eb, (size_t)RpB); r |= dalloc(h, &h->err, 1);
    if (r) return ALFGPU_ERROR_CUDA;
    CK(cudaMemcpy2D(dA, (size_t)m * sizeof(double), A, (size_t)lda * sizeof(double), (size_t)m * sizeof(double), k,
                    cudaMemcpyHostToDevice));
    CK(cudaMemcpy2D(dB, (size_t)k * sizeof(double), B, (size_t)ldb * sizeof(double), (size_t)k * sizeof(double), n,
                    cudaMemcpyHostToDevice));
    CUtensorMap ta, tb;
    if (oz_tmap(&ta, sa, Kp, (long long)S * RpA, OZ_BM) || oz_tmap(&tb, sb, Kp, (long long)S * RpB, bn))
      return ALFGPU_ERROR_CUDA;
    const size_t sm = oz_smem_bytes(bn, S, Kp / OZ_KC, nst);
    if (bn == 32) CK(raise_smem_limit(k_oz_gemm<32>, sm));
    else CK(raise_smem_limit(k_oz_gemm<16>, sm));
    RET(oz_slice(h, dA, OZ_REAL, 1, m, 0, 0, nullptr, 0, m, k, nullptr, S, bits, RpA, Kp, sa, ea, 1));
    RET(oz_slice(h, dB, OZ_REAL, k, 1, 0, 0, nullptr, 0, n, k, nullptr, S, bits, RpB, Kp, sb, eb, 1));
    RET(oz_gemm(h, ta, tb, m, n, Kp, S, bits, bn, nst, RpA, RpB, 0, 0, ea, eb, OZ_OUT_REAL, 0, dC, 1, m, 0, 1));
    RET(check_err(h));
    CK(cudaMemcpy2D(C, (size_t)ldc * sizeof(double), dC, (size_t)m * sizeof(double), (size_t)m * sizeof(double), n,
                    cudaMemcpyDeviceToHost));
    return 0;
  };
  rc = run();
  alfgpu_destroy(h);
  return rc;
}

const char* alfgpu_last_error(alfgpu_t* h) {
  if (!h) return "null handle";
  snprintf(h->last_msg, sizeof(h->last_msg), "alfgpu.cu:%d: %s", h->last_line, cudaGetErrorString(h->last_cuda));
  return h->last_msg;
}

int alfgpu_set_scalar_obs(alfgpu_t* h, const double* H, const double* U) {
  if (!h) return ALFGPU_ERROR_ARGUMENT;
  CK(cudaSetDevice(h->dev));
  if (!H || !U) {  // off
    h->obs_scal = 0;
    drop_graphs(h);
    return 0;
  }
  const size_t N = h->N, NN = N * N, F = h->F;
  if (!h->obs_HT) {
    int r = 0;
    r |= dalloc(h, &h->obs_HT, F * NN); r |= dalloc(h, &h->obs_trH, F); r |= dalloc(h, &h->obs_U, N);
    r |= dalloc(h, &h->obs_acc, 10 * (size_t)h->C);
    if (r) return ALFGPU_ERROR_CUDA;
  }
  std::vector<double> ht(F * NN), tr(F, 0.0);
  for (size_t f = 0; f < F; ++f)
    for (size_t i = 0; i < N; ++i) {
      tr[f] += H[f * NN + i + i * N];
      for (size_t j = 0; j < N; ++j) {
        const double v = H[f * NN + i + j * N];  // H_f(i, j)
        if (!std::isfinite(v)) return ALFGPU_ERROR_ARGUMENT;
        ht[f * NN + j + i * N] = v;
      }
    }
  for (size_t i = 0; i < N; ++i)
    if (!std::isfinite(U[i])) return ALFGPU_ERROR_ARGUMENT;
  if (h->rot) return ALFGPU_ERROR_UNSUPPORTED;  // two-site vertices: measure through the callback
  CK(cudaMemcpy(h->obs_HT, ht.data(), F * NN * sizeof(double), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(h->obs_trH, tr.data(), F * sizeof(double), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(h->obs_U, U, N * sizeof(double), cudaMemcpyHostToDevice));
  CK(cudaMemset(h->obs_acc, 0, 10 * (size_t)h->C * sizeof(double)));
  h->obs_nsun = h->NSUN;
  h->obs_scal = 1;
  drop_graphs(h);
  return 0;
}

int alfgpu_get_scalar_obs(alfgpu_t* h, int32_t chain, double* sums) {
  if (!h || !sums || chain < 0 || chain >= h->C || !h->obs_acc) return ALFGPU_ERROR_ARGUMENT;
  CK(cudaSetDevice(h->dev));
  CK(cudaStreamSynchronize(h->st));
  CK(cudaMemcpy(sums, h->obs_acc + 10ll * chain, 10 * sizeof(double), cudaMemcpyDeviceToHost));
  return 0;
}

int alfgpu_reset_scalar_obs(alfgpu_t* h) {
  if (!h || !h->obs_acc) return ALFGPU_ERROR_ARGUMENT;
  CK(cudaSetDevice(h->dev));
  CK(cudaMemsetAsync(h->obs_acc, 0, 10 * (size_t)h->C * sizeof(double), h->st));
  CK(cudaStreamSynchronize(h->st));
  return 0;
}

// ---- device-side lattice-resolved observables ----------------------------------------------
int alfgpu_set_lattice_obs(alfgpu_t* h, int32_t ncell, int32_t norb, const int32_t* site_of, const int32_t* jof) {
  if (!h) return ALFGPU_ERROR_ARGUMENT;
  CK(cudaSetDevice(h->dev));
  if (!site_of || !jof) {  // off
    h->obs_latt = 0;
    drop_graphs(h);
    return 0;
  }
  if (ncell < 1 || norb < 1 || (long long)ncell * norb != h->N) return ALFGPU_ERROR_ARGUMENT;
  std::vector<int> seen(h->N, 0);
  for (long long e = 0; e < (long long)ncell * norb; ++e) {
    if (site_of[e] < 0 || site_of[e] >= h->N || seen[site_of[e]]) return ALFGPU_ERROR_ARGUMENT;
    seen[site_of[e]] = 1;
  }
  for (int I = 0; I < ncell; ++I) {
    std::vector<int> cs(ncell, 0);
    for (int R = 0; R < ncell; ++R) {
      const int J = jof[(long long)I * ncell + R];
      if (J < 0 || J >= ncell || cs[J]) return ALFGPU_ERROR_ARGUMENT;
      cs[J] = 1;
    }
  }
  const int nnames = h->F == 2 ? 5 : 3;
  if (h->obs_latt || h->lo_site) {
    if (ncell != h->lo_ncell || norb != h->lo_norb) return ALFGPU_ERROR_ARGUMENT;  // one lattice per handle
  } else {
    const size_t C = h->C, no2 = (size_t)norb * norb;
    int r = 0;
    r |= dalloc(h, &h->lo_site, (size_t)ncell * norb); r |= dalloc(h, &h->lo_jof, (size_t)ncell * ncell);
    r |= dalloc(h, &h->lo_acc[0], C * nnames * ncell * no2); r |= dalloc(h, &h->lo_acc0[0], C * nnames * norb);
    r |= dalloc(h, &h->lo_cnt[0], 2 * C);
    if (h->ltau) {
      r |= dalloc(h, &h->lo_acc[1], C * nnames * ncell * (size_t)(h->L + 1) * no2);
      r |= dalloc(h, &h->lo_acc0[1], C * nnames * norb); r |= dalloc(h, &h->lo_cnt[1], 2 * C);
      if (!h->Gq) r |= dalloc(h, &h->Gq, 4 * (size_t)h->B * h->N * h->N);
    }
    if (r) return ALFGPU_ERROR_CUDA;
  }
  h->lo_ncell = ncell; h->lo_norb = norb; h->lo_nnames = nnames;
  CK(cudaMemcpy(h->lo_site, site_of, (size_t)ncell * norb * sizeof(int), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(h->lo_jof, jof, (size_t)ncell * ncell * sizeof(int), cudaMemcpyHostToDevice));
  h->obs_latt = 1;
  drop_graphs(h);
  return alfgpu_reset_lattice_obs(h);
}

int alfgpu_reset_lattice_obs(alfgpu_t* h) {
  if (!h || !h->lo_site) return ALFGPU_ERROR_ARGUMENT;
  CK(cudaSetDevice(h->dev));
  const size_t C = h->C, no2 = (size_t)h->lo_norb * h->lo_norb, nn = h->lo_nnames;
  for (int k = 0; k < 2; ++k) {
    if (!h->lo_acc[k]) continue;
    const size_t L1 = k ? (size_t)h->L + 1 : 1;
    CK(cudaMemsetAsync(h->lo_acc[k], 0, C * nn * h->lo_ncell * L1 * no2 * sizeof(zd), h->st));
    CK(cudaMemsetAsync(h->lo_acc0[k], 0, C * nn * h->lo_norb * sizeof(zd), h->st));
    CK(cudaMemsetAsync(h->lo_cnt[k], 0, 2 * C * sizeof(double), h->st));
  }
  CK(cudaStreamSynchronize(h->st));
  return 0;
}

int alfgpu_get_lattice_obs(alfgpu_t* h, int32_t chain, int32_t kind, double* latt, double* latt0, double* cnt) {
  if (!h || !h->lo_site || chain < 0 || chain >= h->C || kind < 0 || kind > 1 || !h->lo_acc[kind])
    return ALFGPU_ERROR_ARGUMENT;
  CK(cudaSetDevice(h->dev));
  CK(cudaStreamSynchronize(h->st));
  const size_t no2 = (size_t)h->lo_norb * h->lo_norb, nn = h->lo_nnames;
  const size_t L1 = kind ? (size_t)h->L + 1 : 1;
  const size_t n = nn * h->lo_ncell * L1 * no2, n0 = nn * h->lo_norb;
  if (latt) CK(cudaMemcpy(latt, h->lo_acc[kind] + chain * n, n * sizeof(zd), cudaMemcpyDeviceToHost));
  if (latt0) CK(cudaMemcpy(latt0, h->lo_acc0[kind] + chain * n0, n0 * sizeof(zd), cudaMemcpyDeviceToHost));
  if (cnt) CK(cudaMemcpy(cnt, h->lo_cnt[kind] + 2 * chain, 2 * sizeof(double), cudaMemcpyDeviceToHost));
  return 0;
}

// ---- checkerboard hopping ------------------------------------------------------------------
int alfgpu_upload_checkerboard(alfgpu_t* h, int32_t ncheck, int32_t nfam, const int32_t* fam, const int32_t* P,
                               const double* mat, const double* inv) {
  if (!h || ncheck < 0 || (ncheck > 0 && (!fam || !P || !mat || !inv || nfam < 1))) return ALFGPU_ERROR_ARGUMENT;
  CK(cudaSetDevice(h->dev));
  if (ncheck == 0) {  // back to the dense exponentials of alfgpu_upload_hopping
    h->cb = 0;
    drop_graphs(h);
    return 0;
  }
  if (h->rot) return ALFGPU_ERROR_UNSUPPORTED;  // bonds in the rotated basis of two-site vertices: not built
  const int N = h->N, F = h->F;
  if (fam[0] != 0 || fam[nfam] != ncheck) return ALFGPU_ERROR_ARGUMENT;
  for (int q = 0; q < nfam; ++q) {
    if (fam[q + 1] < fam[q]) return ALFGPU_ERROR_ARGUMENT;
    for (int f = 0; f < F; ++f) {  // the bonds of a family are disjoint
      std::vector<int> seen(N, 0);
      for (int nc = fam[q]; nc < fam[q + 1]; ++nc)
        for (int e = 0; e < 2; ++e) {
          const int s = P[2 * ((size_t)f * ncheck + nc) + e];
          if (s < 0 || s >= N || seen[s]) return ALFGPU_ERROR_HAMILTONIAN;
          seen[s] = 1;
        }
    }
  }
  for (size_t k = 0; k < 4ull * F * ncheck; ++k)
    if (!std::isfinite(mat[k]) || !std::isfinite(inv[k])) return ALFGPU_ERROR_HAMILTONIAN;
  if (ncheck > h->cb_ncheck) {
    int r = 0;
    r |= dalloc(h, &h->cb_P, 2ull * F * ncheck);
    r |= dalloc(h, &h->cb_mat, 4ull * F * ncheck); r |= dalloc(h, &h->cb_inv, 4ull * F * ncheck);
    if (r) return ALFGPU_ERROR_CUDA;
  }
  CK(cudaMemcpy(h->cb_P, P, 2ull * F * ncheck * sizeof(int), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(h->cb_mat, mat, 4ull * F * ncheck * sizeof(double), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(h->cb_inv, inv, 4ull * F * ncheck * sizeof(double), cudaMemcpyHostToDevice));
  h->cb_ncheck = ncheck;
  h->cb_fam.assign(fam, fam + nfam + 1);
  h->cb = 1;
  drop_graphs(h);
  return 0;
}
