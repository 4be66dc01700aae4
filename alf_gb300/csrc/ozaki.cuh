// FP64-accurate real GEMM on the BF16 tensor cores (tcgen05 + TMA), by exact digit
// slicing (the Ozaki scheme: T. Ozaki, T. Ogita, S. Oishi, S. M. Rump, "Error-free
// transformations of matrix multiplication by using fast routines of matrix
// multiplication and its applications", Numer. Algorithms 59, 2012).
//
// Every row of the M-side operand A (and every row of the N-side operand B, i.e. every
// output column) is scaled by a power of two 2^-e with |x| < 2^e over the row, and its
// entries are cut into S signed digits of b bits, x = 2^e sum_s d_s 2^(-b s),
// |d_s| < 2^b.  The digits are integers, exact in BF16 (b <= 7).  For each anti-diagonal
// D = s + t <= S + 2 of the digit products, sum_{s+t=D} A_s B_t is accumulated on the
// tensor cores in FP32; b and S are chosen so that every partial sum is an integer below
// 2^24, so these accumulations are exact.  The diagonals are combined in 64-bit integer
// arithmetic and rounded once to FP64.  With S b >= 54 the product carries an error below
// 2^-53 (max_k |A_ik|) (sum_k |B_kj|) + 2^-53 (max_k |B_kj|) (sum_k |A_ik|) (operand
// truncation; the dropped diagonals D >= S + 3 add < 2^-56 K max|A_i.| max|B_.j|), i.e.
// FP64-level on the O(1) entries of Green functions and hopping exponentials; FP32
// products (2^-24) are not enough there (they are amplified by the stabilisation
// interval).  Complex products are real GEMMs on interleaved real/imaginary rows
// (k_oz_slice modes) with the complex element assembled in the epilogue.  The first S'
// digits of an S-digit slicing are the S'-digit slicing of the same element (same row
// exponent and digit width), so a product may use a prefix of a buffer's slices (SbA /
// SbB give the buffers' own slice counts): fewer slices trade accuracy, 2^-(b S'), for
// (S' + 1)(S' + 2)/2 - 2 instead of (S + 1)(S + 2)/2 - 2 digit products.
//
//   k_oz_slice  FP64 -> BF16 digit slices [batch][S][Rpad][Kpad] (K contiguous) and the
//               row exponents, integer arithmetic only (the FP64 pipe is 1/64 of FP32)
//   k_oz_gemm   one CTA per 128 x BN output tile: all B slices of the tile resident in
//               shared memory (TMA, 128-byte swizzle), A slices streamed through a ring of
//               64-wide K chunks by a producer warp; an MMA warp issues, per A slice and
//               K step, one tcgen05.mma (M = 128, N = up to 256, K = 16, BF16 -> FP32)
//               against all B slices at once, into S + 1 TMEM accumulators (one per
//               diagonal, the MMA's column base offset by the A slice index), and
//               tcgen05.commit releases ring stages; eight warps read TMEM back
//               (tcgen05.ld 32x32b), combine, round, and write complex128/float64.
#pragma once
#include <cuda.h>
#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>

#include "common.cuh"

enum { OZ_REAL = 0, OZ_CROWS = 1, OZ_CKA = 2, OZ_CKB = 3 };
enum { OZ_OUT_COLS = 0, OZ_OUT_ROWS = 1, OZ_OUT_REAL = 2, OZ_OUT_CPLX = 3 };
#define OZ_KC 64          // K chunk of one TMA box (128 bytes of BF16)
#define OZ_BM 128         // MMA M
#ifndef OZ_TARGET_BITS
#define OZ_TARGET_BITS 54  // digits x bits per slice >= this (an FP64 mantissa and one guard bit)
#endif

// ---------------------------------------------------------------------------------------
// Slicing
// ---------------------------------------------------------------------------------------
struct OzSliceParams {
  const void* src;          // complex128 (OZ_C*) or float64 (OZ_REAL)
  int mode;                 // OZ_*
  long long sr, sk, sb;     // source element strides: row, k, batch
  int modb;                 // source batch = b % modb when > 0
  const zd* ks; long long sks;  // optional real per-k scale (real part; complex k index)
  int conj;                 // OZ_CROWS: negate imaginary parts
  int srows;                // source rows (complex rows for OZ_C*)
  int Kc;                   // source K extent (complex k for OZ_C*)
  const int* kdyn;          // optional per-batch valid source K (entries beyond are zero)
  const int* perm; long long sperm;  // optional K remap (OZ_CROWS): element (i, k) is source (i, perm[k])
  int tri, trans;           // tri: zero the strictly lower triangle of the source in storage
                            // coordinates (row, col) = trans ? (k', i) : (i, k'), k' the remapped k
  const zd* rsc; long long srsc; int rinv;  // optional real per-row scale (real part), or its inverse
  int kvalid;               // > 0: source k >= kvalid are zero (with kdyn: the smaller bound)
  int unitlow, doff;        // OZ_CROWS: the source is a unit lower trapezoid (Householder vectors of a
                            // QR panel): storage (r, c) is 0 for r < c + doff, 1 for r == c + doff
  int S, bits;
  int Rpad, Kpad;
  unsigned short* out;      // BF16 bits, [batch][S][Rpad][Kpad]
  int* expo;                // [batch][Rpad]
  int* err;                 // bit 0: non-finite input
};

struct OzNum {
  unsigned long long m;  // value = (-1)^neg m 2^e2; m == 0: zero
  int e2, neg;
};

ALF_DEV OzNum oz_decode(double x, int* bad) {
  const unsigned long long u = (unsigned long long)__double_as_longlong(x);
  const int E = (int)((u >> 52) & 0x7ff);
  OzNum r;
  r.neg = (int)(u >> 63);
  if (E == 0 || E == 0x7ff) {  // zero, subnormal (below 2^-1022: 0 here), inf / NaN (flagged)
    if (E == 0x7ff) *bad = 1;
    r.m = 0; r.e2 = 0;
    return r;
  }
  r.m = ((u & 0xfffffffffffffull) | 0x10000000000000ull) << 11;
  r.e2 = E - 1086;
  return r;
}

// x s as (m, e2, neg) with the product of the two 64-bit mantissas truncated to its high
// word (error < 2^-62 relative); s == nullptr: x alone.
ALF_DEV OzNum oz_num(double x, const double* s, int* bad) {
  OzNum n = oz_decode(x, bad);
  if (s && n.m) {
    const OzNum t = oz_decode(*s, bad);
    if (!t.m) { n.m = 0; return n; }
    n.m = __umul64hi(n.m, t.m);  // >= 2^62
    n.e2 += t.e2 + 64;
    n.neg ^= t.neg;
  }
  return n;
}



// Upper bound e with |x s| < 2^e from the exponent fields alone (one above the tight bound
// when the mantissa product stays below 2); x or s zero: -100000.
ALF_DEV int oz_ebound(double x, const double* s) {
  const int ex = (int)((__double_as_longlong(x) >> 52) & 0x7ff);
  if (ex == 0 || ex == 0x7ff) return -100000;
  int e = ex - 1022;
  if (s) {
    const int es = (int)((__double_as_longlong(*s) >> 52) & 0x7ff);
    if (es == 0 || es == 0x7ff) return -100000;
    e += es - 1022;
  }
  return e;
}

// BF16 bits of the integer d, |d| < 2^22 (exact for |d| < 256): d + 1.5 2^23 in FP32 is
// exact, subtracting the bias leaves (float)d, whose low 16 bits are zero.
ALF_DEV unsigned oz_bf16_bits(int d) {
  const float f = __int_as_float(0x4B400000 + d) - 12582912.0f;
  return (unsigned)__float_as_int(f) >> 16;
}

// Digits of one element pair of one logical row, one 32-bit word (two BF16) per slice.
ALF_DEV void oz_write_pair(const OzSliceParams& p, unsigned* o, double x0, double x1, const double* s0,
                           const double* s1, int e, int* bad) {
  const int bS = p.bits * p.S;
  const unsigned mask = (1u << p.bits) - 1u;
  const size_t sstride = (size_t)p.Rpad * p.Kpad / 2;
  unsigned long long v[2];
  int ng[2];
  const double xs[2] = {x0, x1};
  const double* ss[2] = {s0, s1};
#pragma unroll
  for (int u = 0; u < 2; ++u) {
    const OzNum n = oz_num(xs[u], ss[u], bad);
    ng[u] = n.neg;
    v[u] = 0ull;
    if (n.m) {
      const int sh = n.e2 + bS - e;  // |x s| 2^(bS - e) < 2^bS
      v[u] = sh >= 0 ? (sh >= 64 ? 0ull : n.m << sh) : (-sh >= 64 ? 0ull : n.m >> (-sh));
    }
  }
  const unsigned l0 = (unsigned)v[0], h0 = (unsigned)(v[0] >> 32);
  const unsigned l1 = (unsigned)v[1], h1 = (unsigned)(v[1] >> 32);
  for (int s = 0; s < p.S; ++s) {
    const int sh = p.bits * (p.S - 1 - s);
    const unsigned a = sh >= 32 ? (h0 >> (sh - 32)) : __funnelshift_r(l0, h0, sh);
    const unsigned c = sh >= 32 ? (h1 >> (sh - 32)) : __funnelshift_r(l1, h1, sh);
    int d0 = (int)(a & mask), d1 = (int)(c & mask);
    if (ng[0]) d0 = -d0;
    if (ng[1]) d1 = -d1;
    o[(size_t)s * sstride] = oz_bf16_bits(d0) | (oz_bf16_bits(d1) << 16);
  }
}

// One CTA per source row (one or two logical rows), one thread per pair of consecutive k:
// the row exponent(s) by a block reduction of exponent-field bounds, then the S digits of
// both elements of the pair (K contiguous).  Logical rows: OZ_REAL row i; OZ_CROWS 2 i + c
// (c = 0 real, 1 imaginary part of source row i); OZ_CKA row i with K = 2 Kc ([Re | Im]);
// OZ_CKB 2 j + c with K = 2 Kc: row 2j [Re Y(:, j); -Im Y(:, j)], row 2j + 1 [Im Y(:, j);
// Re Y(:, j)].  Padding rows of `out` are never written (zero from allocation); every
// k < Kl of a written row is (and k = Kl when Kl is odd), entries beyond kdyn as zeros.
// grid (srows, batch), blockDim = 32 ceil(Kl / 64) <= 256
__global__ void __launch_bounds__(256) k_oz_slice(OzSliceParams p) {
  __shared__ int red[2][8];
  const int b = blockIdx.y, i = blockIdx.x, tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const bool two = p.mode == OZ_CROWS || p.mode == OZ_CKB;
  const int Kl = (p.mode == OZ_CKA || p.mode == OZ_CKB) ? 2 * p.Kc : p.Kc;
  const int bs = p.modb > 0 ? b % p.modb : b;
  const double* srd = (const double*)p.src + (size_t)bs * p.sb;
  const zd* srz = (const zd*)p.src + (size_t)bs * p.sb;
  const zd* ks = p.ks ? p.ks + (size_t)b * p.sks : nullptr;
  int kd = p.kdyn ? min(p.kdyn[b], p.Kc) : p.Kc;
  if (p.kvalid > 0) kd = min(kd, p.kvalid);
  double x0[2] = {0.0, 0.0}, x1[2] = {0.0, 0.0}, sc[2] = {1.0, 1.0};
  const int k0 = 2 * tid;
  double rs_row = 1.0;  // per-row scale (an output row / column scale of the product)
  if (p.rsc) {
    rs_row = p.rsc[(size_t)b * p.srsc + i].x;
    if (p.rinv) rs_row = 1.0 / rs_row;
  }
  const bool scaled = ks != nullptr || p.rsc != nullptr;
#pragma unroll
  for (int u = 0; u < 2; ++u) {
    const int k = k0 + u;
    if (k >= Kl) continue;
    switch (p.mode) {
      case OZ_REAL:
        if (k < kd) x0[u] = srd[i * p.sr + k * p.sk];
        break;
      case OZ_CROWS:
        if (k < kd) {
          const int kq = p.perm ? p.perm[(size_t)b * p.sperm + k] : k;
          if (p.tri && (p.trans ? kq > i : i > kq)) break;  // below the diagonal of an upper triangle
          if (p.unitlow) {
            const int r = p.trans ? kq : i, cc = (p.trans ? i : kq) + p.doff;
            if (r < cc) break;
            if (r == cc) { x0[u] = 1.0; break; }
          }
          const zd z = srz[i * p.sr + kq * p.sk];
          x0[u] = z.x; x1[u] = p.conj ? -z.y : z.y;
        }
        break;
      case OZ_CKA: {
        const int kc = k < p.Kc ? k : k - p.Kc;
        if (kc < kd) { const zd z = srz[i * p.sr + kc * p.sk]; x0[u] = k < p.Kc ? z.x : z.y; }
      } break;
      default: {
        const int kc = k < p.Kc ? k : k - p.Kc;
        if (kc < kd) {
          const zd z = srz[i * p.sr + kc * p.sk];
          x0[u] = k < p.Kc ? z.x : -z.y;
          x1[u] = k < p.Kc ? z.y : z.x;
        }
      } break;
    }
    if (ks) sc[u] = ks[k].x;
    if (p.rsc) sc[u] = rs_row;
  }
  int e0 = max(oz_ebound(x0[0], scaled ? &sc[0] : nullptr), oz_ebound(x0[1], scaled ? &sc[1] : nullptr));
  int e1 = two ? max(oz_ebound(x1[0], scaled ? &sc[0] : nullptr), oz_ebound(x1[1], scaled ? &sc[1] : nullptr))
               : -100000;
  e0 = __reduce_max_sync(0xffffffffu, e0);
  e1 = __reduce_max_sync(0xffffffffu, e1);
  if (lane == 0) { red[0][warp] = e0; red[1][warp] = e1; }
  __syncthreads();
  const int nw = blockDim.x >> 5;
  for (int w = 0; w < nw; ++w) { e0 = max(e0, red[0][w]); e1 = max(e1, red[1][w]); }
  if (e0 == -100000) e0 = 0;
  if (e1 == -100000) e1 = 0;
  const int r0 = two ? 2 * i : i;
  if (tid == 0) {
    p.expo[(size_t)b * p.Rpad + r0] = e0;
    if (two) p.expo[(size_t)b * p.Rpad + r0 + 1] = e1;
  }
  if (k0 >= Kl) return;
  int bad = 0;
  unsigned* o = reinterpret_cast<unsigned*>(p.out + ((size_t)b * p.S * p.Rpad + r0) * p.Kpad + k0);
  oz_write_pair(p, o, x0[0], x0[1], scaled ? &sc[0] : nullptr, scaled ? &sc[1] : nullptr, e0, &bad);
  if (two)
    oz_write_pair(p, o + p.Kpad / 2, x1[0], x1[1], scaled ? &sc[0] : nullptr, scaled ? &sc[1] : nullptr, e1, &bad);
  if (bad && p.err) atomicOr(p.err, 1);
}

static inline cudaError_t oz_launch_slice(const OzSliceParams& p, int batch, cudaStream_t st) {
  const int Kl = (p.mode == OZ_CKA || p.mode == OZ_CKB) ? 2 * p.Kc : p.Kc;
  if (Kl > 512) return cudaErrorInvalidValue;
  k_oz_slice<<<dim3(p.srows, batch), 32 * ((Kl + 63) / 64), 0, st>>>(p);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------------------
// tcgen05 / TMA / mbarrier primitives
// ---------------------------------------------------------------------------------------
ALF_DEV uint32_t oz_smem(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

ALF_DEV void oz_mbar_init(uint32_t bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}
ALF_DEV void oz_mbar_expect_tx(uint32_t bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}
ALF_DEV bool oz_mbar_try(uint32_t bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(bar), "r"(parity)
      : "memory");
  return ok != 0;
}
// Bounded wait: gives up after ~2^31 SM cycles (about one second) and returns false.
ALF_DEV bool oz_mbar_wait(uint32_t bar, uint32_t parity) {
  const long long t0 = clock64();
  while (!oz_mbar_try(bar, parity))
    if (clock64() - t0 > (1ll << 31)) return false;
  return true;
}
ALF_DEV void oz_tma_2d(uint32_t dst, const CUtensorMap* tm, int x, int y, uint32_t bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
          dst),
      "l"((unsigned long long)tm), "r"(x), "r"(y), "r"(bar)
      : "memory");
}
// Shared-memory matrix descriptor: K-major operand in the canonical 128-byte-swizzled
// layout (8-row x 128-byte atoms, atoms 1024 bytes apart along M/N), as written by TMA
// with CU_TENSOR_MAP_SWIZZLE_128B.  Fields: start >> 4 [0,14), leading byte offset >> 4
// [16,30) (unused for this layout), stride byte offset >> 4 [32,46), version 1 [46,48),
// swizzle mode 2 = 128 B [61,64).
ALF_DEV uint64_t oz_desc(uint32_t saddr) {
  return (uint64_t)((saddr & 0x3ffffu) >> 4) | ((uint64_t)1 << 16) | ((uint64_t)(1024 >> 4) << 32) |
         ((uint64_t)1 << 46) | ((uint64_t)2 << 61);
}
// Instruction descriptor, kind::f16: FP32 accumulator [4,6) = 1, A and B BF16 [7,10) =
// [10,13) = 1, both K-major, N >> 3 at [17,23), M >> 4 at [24,29).
ALF_DEV uint32_t oz_idesc(int n) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(OZ_BM >> 4) << 24);
}
ALF_DEV void oz_mma(uint32_t dtmem, uint64_t ad, uint64_t bd, uint32_t idesc, uint32_t acc) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(dtmem),
      "l"(ad), "l"(bd), "r"(idesc), "r"(acc)
      : "memory");
}
ALF_DEV void oz_commit(uint32_t bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar) : "memory");
}
ALF_DEV void oz_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
ALF_DEV void oz_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }

template <int BN>
ALF_DEV void oz_tmem_ld(uint32_t taddr, uint32_t (&r)[BN]);
template <>
ALF_DEV void oz_tmem_ld<32>(uint32_t taddr, uint32_t (&r)[32]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
      "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
        "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
        "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}
template <>
ALF_DEV void oz_tmem_ld<16>(uint32_t taddr, uint32_t (&r)[16]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

template <>
ALF_DEV void oz_tmem_ld<8>(uint32_t taddr, uint32_t (&r)[8]) {
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
               : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

// An FP32 value that holds an integer of magnitude < 2^31, as int (bit manipulation on the
// integer pipes).
ALF_DEV int oz_f2i(uint32_t u) {
  const int e = (int)((u >> 23) & 0xff);
  if (e < 127) return 0;  // |x| < 1: the exact integer sum is 0
  const int m = (int)((u & 0x7fffffu) | 0x800000u);
  const int sh = 150 - e;
  const int v = sh >= 0 ? (m >> sh) : (sh > -8 ? (m << -sh) : 0x7fffffff);
  return (u >> 31) ? -v : v;
}

// z 2^sc rounded to the nearest FP64 (ties to even), integer arithmetic only.
ALF_DEV double oz_i64_to_f64(long long z, int sc) {
  if (z == 0) return 0.0;
  const unsigned long long sgn = z < 0 ? (1ull << 63) : 0ull;
  const unsigned long long a = z < 0 ? (unsigned long long)(-z) : (unsigned long long)z;
  const int p = 63 - __clzll((long long)a);
  unsigned long long m;
  int e = p + sc;
  if (p > 52) {
    const int r = p - 52;
    m = a >> r;
    const unsigned long long rem = a & ((1ull << r) - 1), half = 1ull << (r - 1);
    if (rem > half || (rem == half && (m & 1))) {
      ++m;
      if (m >> 53) { m >>= 1; ++e; }
    }
  } else {
    m = a << (52 - p);
  }
  const int be = e + 1023;
  if (be <= 0) return __longlong_as_double((long long)sgn);
  if (be >= 2047) return __longlong_as_double((long long)(sgn | 0x7ff0000000000000ull));
  return __longlong_as_double((long long)(sgn | ((unsigned long long)be << 52) | (m & 0xfffffffffffffull)));
}

// ---------------------------------------------------------------------------------------
// GEMM
// ---------------------------------------------------------------------------------------
struct OzGemmParams {
  int M, N;                  // logical rows of A and of B (valid extents)
  int nkc, S, bits, nst;     // K chunks (Kpad / 64), slices, bits per slice, ring stages
  int nd;                    // diagonals accumulated: s + t < nd (0-based digit indices)
  int L;                     // fixed-point position of the combined integer (oz_shift)
  int RpadA, RpadB;
  int modA, modB;            // operand batch = b % mod when > 0
  const int* expA; const int* expB;
  int omode, osub;           // OZ_OUT_*; osub 1: out -= A B, -1: out += A B (OZ_OUT_CPLX)
  void* out; long long ldr, ldc, sout;  // element strides (complex128 for _COLS/_ROWS, float64 for _REAL)
  int* err;                  // bit 2: a bounded wait gave up
  const zd* rsc; long long srsc;  // optional real scale of output row m (real part used), per batch
  const zd* csc; long long scsc;  // optional real scale of output column n (OZ_OUT_ROWS; real part), per batch
  int SbA, SbB;              // slices per batch entry in the A / B slice buffers (>= S: the first S are used)
  // k_oz_gemm<BN, true>: the grid is smaller than the tile count and each CTA takes tiles
  // blockIdx.x, blockIdx.x + gridDim.x, ... of the tiles_n x tiles_m x tiles_b tiles (N-tile
  // fastest); <BN, false>: one tile per CTA at (blockIdx.x, blockIdx.y, blockIdx.z)
  int persist, tiles_n, tiles_m, tiles_b;
};

static inline size_t oz_smem_bytes(int bn, int S, int nkc, int nst) {
  return (size_t)(S + 1) * nkc * bn * 128 + (size_t)nst * OZ_BM * 128 + 256 + 1024;
}

// 256 threads.  Warp 0 lane 0 is the TMA producer (B slices once, A chunks into the ring
// as stages free up), warp 1 lane 0 issues the MMAs and commits each ring stage back to the
// producer; then all eight warps read TMEM: warp w takes TMEM lanes 32 (w % 4) .. + 31
// (its sub-partition's) and columns (w / 4) BN/2 .. + BN/2 - 1.
template <int BN, bool PERSIST = false>
__global__ void __launch_bounds__(256, 1) k_oz_gemm(const __grid_constant__ CUtensorMap tmA,
                                                    const __grid_constant__ CUtensorMap tmB, OzGemmParams p) {
  constexpr int HB = BN / 2;  // columns per epilogue thread
  extern __shared__ unsigned char oz_raw[];
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int S = p.S, nkc = p.nkc, NST = p.nst, ND = p.nd;
  const uint32_t raw = oz_smem(oz_raw);
  const uint32_t base = (raw + 1023u) & ~1023u;
  const uint32_t sB = base;                                     // [nkc][S + 1][BN rows x 128 B], block S zero
  const uint32_t sA = sB + (uint32_t)((S + 1) * nkc * BN * 128);  // [NST][128 rows x 128 B]
  const uint32_t sBar = sA + (uint32_t)(NST * OZ_BM * 128);     // full[NST], empty[NST], bfull, done
  unsigned char* gbar = oz_raw + (sBar - raw);
  const uint32_t full0 = sBar, empty0 = sBar + 8u * NST, bfull = sBar + 16u * NST, done = bfull + 8;
  uint32_t* tslot = reinterpret_cast<uint32_t*>(gbar + 16 * NST + 16);
  volatile int* abort_flag = reinterpret_cast<volatile int*>(gbar + 16 * NST + 20);
  volatile int* consumed_sh = reinterpret_cast<volatile int*>(gbar + 16 * NST + 24);
  int ncols = 32;
  while (ncols < ND * BN) ncols <<= 1;

  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(oz_smem(tslot)),
                 "r"(ncols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  if (tid == 32) {
    for (int i = 0; i < NST; ++i) { oz_mbar_init(full0 + 8u * i, 1); oz_mbar_init(empty0 + 8u * i, 1); }
    oz_mbar_init(bfull, 1);
    oz_mbar_init(done, 1);
    *abort_flag = 0;
    *consumed_sh = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  }
  for (int kc = 0; kc < nkc; ++kc) {  // block t = S of every K chunk: zeros (read by the s = 0 MMAs)
    uint4* z = reinterpret_cast<uint4*>(oz_raw + (sB - raw) + (size_t)(kc * (S + 1) + S) * BN * 128);
    for (int i = tid; i < BN * 8; i += 256) z[i] = make_uint4(0u, 0u, 0u, 0u);
  }
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");  // generic writes -> tensor-core reads
  oz_fence_before();
  __syncthreads();
  oz_fence_after();
  const uint32_t tbase = *tslot;
  const int total = S * nkc;
  const uint32_t chunkA = OZ_BM * 128, chunkB = BN * 128;
  const int ntile = PERSIST ? p.tiles_n * p.tiles_m * p.tiles_b : 1;
  // ring stage and round of a chunk follow its count over all tiles of this CTA, kept as running
  // (stage, round) pairs by the producer and the MMA issuer; bfull and done complete once per
  // tile (parity = tile iteration & 1)
  int pst = 0, pround = 0, mst = 0, mround = 0;
  int it = 0;
  // A-resident mode (persistent, every A chunk of a tile fits the ring): a CTA takes a contiguous
  // range of tiles, N-tile fastest, so consecutive tiles share their A chunks, which are loaded
  // into stages 0 .. total - 1 only when the (batch, M-tile) changes; the ring's empty barriers
  // are not used (the previous tile's MMAs are complete before the next tile starts)
  const bool resident = PERSIST && total <= NST;
  int t_begin = 0, t_end = 1, t_step = 1;
  if (PERSIST && resident) {
    t_begin = (int)((long long)ntile * blockIdx.x / gridDim.x);
    t_end = (int)((long long)ntile * (blockIdx.x + 1) / gridDim.x);
  } else if (PERSIST) {
    t_begin = (int)blockIdx.x; t_end = ntile; t_step = (int)gridDim.x;
  }
  int keyA_prev = -1, aloads = 0;
  for (int tix = t_begin; tix < t_end; tix += t_step, ++it) {
  int b, m0, n0;
  if (PERSIST) {
    n0 = (tix % p.tiles_n) * BN;
    m0 = ((tix / p.tiles_n) % p.tiles_m) * OZ_BM;
    b = tix / (p.tiles_n * p.tiles_m);
  } else {
    b = blockIdx.z; m0 = blockIdx.y * OZ_BM; n0 = blockIdx.x * BN;
  }
  const int bA = p.modA > 0 ? b % p.modA : b, bB = p.modB > 0 ? b % p.modB : b;
  const int g0 = it * total;  // count of this tile's first A chunk
  const uint32_t tpar = (uint32_t)(it & 1);
  const int keyA = bA * p.tiles_m + m0 / OZ_BM;
  const bool loadA = !resident || keyA != keyA_prev;
  if (resident && loadA) { keyA_prev = keyA; ++aloads; }
  const uint32_t apar = (uint32_t)((aloads - 1) & 1);  // resident A: parity of its load

  if (tid == 0) {  // producer
    const int rowA0 = bA * p.SbA * p.RpadA + m0, rowB0 = bB * p.SbB * p.RpadB + n0;
    oz_mbar_expect_tx(bfull, (uint32_t)(S * nkc) * chunkB);
    for (int t = 0; t < S; ++t)
      for (int kc = 0; kc < nkc; ++kc)
        oz_tma_2d(sB + (uint32_t)(kc * (S + 1) + t) * chunkB, &tmB, kc * OZ_KC, rowB0 + t * p.RpadB, bfull);
    int loaded = 0;
    bool ok = true;
    if (resident) {
      if (loadA)
        for (int l = 0; l < total; ++l) {
          oz_mbar_expect_tx(full0 + 8u * l, chunkA);
          oz_tma_2d(sA + (uint32_t)l * chunkA, &tmA, (l % nkc) * OZ_KC, rowA0 + (l / nkc) * p.RpadA, full0 + 8u * l);
        }
      loaded = total;
    }
    for (int s = 0, kc = 0; !resident && loaded < total; ++loaded) {
      const int st = pst;
      if (pround > 0 && !oz_mbar_wait(empty0 + 8u * st, (uint32_t)((pround - 1) & 1))) { ok = false; break; }
      if (*abort_flag) break;
      oz_mbar_expect_tx(full0 + 8u * st, chunkA);
      oz_tma_2d(sA + (uint32_t)st * chunkA, &tmA, kc * OZ_KC, rowA0 + s * p.RpadA, full0 + 8u * st);
      if (++pst == NST) { pst = 0; ++pround; }
      if (++kc == nkc) { kc = 0; ++s; }
    }
    if (!ok) { atomicOr(p.err, 4); *abort_flag = 1; }
    if (*abort_flag) {  // let every copy issued by this thread land before the CTA exits
      oz_mbar_wait(bfull, tpar);
      if (resident) {
        if (loadA)
          for (int l = 0; l < total; ++l) oz_mbar_wait(full0 + 8u * l, apar);
      } else {
        for (int q = g0 + *consumed_sh; q < g0 + loaded; ++q)
          oz_mbar_wait(full0 + 8u * (uint32_t)(q % NST), (uint32_t)((q / NST) & 1));
      }
    }
  } else if (tid == 32) {  // MMA issuer
    oz_fence_after();  // the previous tile's TMEM reads are done (barrier below)
    bool ok = oz_mbar_wait(bfull, tpar);
    // descriptors differ only in the start-address field: advance them by (bytes >> 4)
    const uint64_t dA0 = oz_desc(sA), dB0 = oz_desc(sB);
    constexpr int TMAX = 256 / BN;  // B blocks per MMA (N <= 256)
    int q = 0;
    for (int s = 0, kc = 0; ok && q < total; ++q) {
      const int st = resident ? q : mst;
      if (!oz_mbar_wait(full0 + 8u * st, resident ? apar : (uint32_t)(mround & 1))) { ok = false; break; }
      oz_fence_after();
      const uint64_t dA = dA0 + (uint64_t)((st * chunkA) >> 4);
      // A_s times the contiguous blocks B_0 .. B_{nt-1} of this K chunk in one MMA (N = nt BN),
      // into TMEM columns (s + t) BN: each product lands in its diagonal's accumulator.  For
      // s = 0 the zero block t = S covers the last diagonal, so every accumulator is written
      // (not accumulated) by the first K step.
      const int nt = ND - s;
      for (int kk = 0; kk < OZ_KC / 16; ++kk) {
        const uint32_t acc = (s == 0 && kc == 0 && kk == 0) ? 0u : 1u;
        for (int t0 = 0; t0 < nt; t0 += TMAX) {
          const int n = min(TMAX, nt - t0);
          const uint64_t dB = dB0 + (uint64_t)(((kc * (S + 1) + t0) * chunkB) >> 4) + 2u * kk;
          oz_mma(tbase + (uint32_t)((s + t0) * BN), dA + 2u * kk, dB, oz_idesc(n * BN), acc);
        }
      }
      if (!resident) {
        oz_commit(empty0 + 8u * st);
        if (++mst == NST) { mst = 0; ++mround; }
      }
      *consumed_sh = q + 1;
      if (++kc == nkc) { kc = 0; ++s; }
    }
    if (!ok) { atomicOr(p.err, 4); *abort_flag = 1; }
    oz_commit(done);  // arrives when every MMA issued above has completed
  }
  __syncwarp();
  const bool done_ok = oz_mbar_wait(done, tpar);
  oz_fence_after();
  __syncthreads();
  if (!done_ok && lane == 0) { atomicOr(p.err, 4); *abort_flag = 1; }
  if (done_ok && !*abort_flag) {
    const int quarter = warp & 3, half = warp >> 2;
    const int c0 = half * HB;  // first tile column of this thread
    long long Z[HB];
#pragma unroll
    for (int j = 0; j < HB; ++j) Z[j] = 0;
    const int L = p.L;
    for (int d = 0; d < ND; ++d) {
      uint32_t r[HB];
      oz_tmem_ld<HB>(tbase + ((uint32_t)(32 * quarter) << 16) + (uint32_t)(d * BN + c0), r);
      const int sh = L - p.bits * (d + 2);
#pragma unroll
      for (int j = 0; j < HB; ++j) {
        const long long v = (long long)oz_f2i(r[j]);
        Z[j] += sh >= 0 ? v * (1ll << sh) : ((v + (1ll << (-sh - 1))) >> (-sh));  // rounded
      }
    }
    const int m = m0 + 32 * quarter + lane;
    const int ea = (m < p.M) ? p.expA[(size_t)bA * p.RpadA + m] : 0;
    double v[HB];
#pragma unroll
    for (int j = 0; j < HB; ++j) {
      const int n = n0 + c0 + j;
      const int eb = (n < p.N) ? p.expB[(size_t)bB * p.RpadB + n] : 0;
      v[j] = oz_i64_to_f64(Z[j], ea + eb - L);
    }
    if (p.rsc && m < p.M) {
      const double s = p.rsc[(size_t)b * p.srsc + m].x;
#pragma unroll
      for (int j = 0; j < HB; ++j) v[j] *= s;
    }
    if (p.csc) {  // OZ_OUT_ROWS: real column n is complex column n
#pragma unroll
      for (int j = 0; j < HB; ++j) {
        const int n = n0 + c0 + j;
        if (n < p.N) v[j] *= p.csc[(size_t)b * p.scsc + n].x;
      }
    }
    if (p.omode == OZ_OUT_REAL) {
      double* o = (double*)p.out + (size_t)b * p.sout;
      if (m < p.M)
#pragma unroll
        for (int j = 0; j < HB; ++j)
          if (n0 + c0 + j < p.N) {
            double* w = o + m * p.ldr + (n0 + c0 + j) * p.ldc;
            *w = p.osub ? *w - v[j] : v[j];
          }
    } else if (p.omode == OZ_OUT_COLS) {  // real column 2 j + c -> complex column j
      zd* o = (zd*)p.out + (size_t)b * p.sout;
      if (m < p.M)
#pragma unroll
        for (int j = 0; j < HB / 2; ++j) {
          const int jc = (n0 + c0) / 2 + j;
          if (2 * jc < p.N) {
            zd* w = o + m * p.ldr + jc * p.ldc;
            zd x = zmk(v[2 * j], v[2 * j + 1]);
            if (p.osub) { const zd g = *w; x = zmk(g.x - x.x, g.y - x.y); }
            *w = x;
          }
        }
    } else if (p.omode == OZ_OUT_CPLX) {
      // complex x complex: rows 2i / 2i+1 hold Re / Im of A's row i, columns 2j / 2j+1 Re / Im
      // of op(B)'s column j; C(i, j) = (ReA ReB - ImA ImB) + i (ReA ImB + ImA ReB).  The lane
      // pair of rows 2i, 2i+1 exchanges halves: even lanes finish the first HQ complex columns
      // of the thread's HB real columns, odd lanes the other HQ.
      zd* o = (zd*)p.out + (size_t)b * p.sout;
      const int i = m >> 1, c = m & 1;
      constexpr int HQ = HB / 4;
      double mine[HB / 2], got[HB / 2];
#pragma unroll
      for (int q2 = 0; q2 < HQ; ++q2) {
        // static register indices: select the value, not the index
        const double lo0 = v[2 * q2], lo1 = v[2 * q2 + 1], hi0 = v[2 * (HQ + q2)], hi1 = v[2 * (HQ + q2) + 1];
        got[2 * q2] = __shfl_xor_sync(0xffffffffu, c ? lo0 : hi0, 1);  // what the partner finishes
        got[2 * q2 + 1] = __shfl_xor_sync(0xffffffffu, c ? lo1 : hi1, 1);
        mine[2 * q2] = c ? hi0 : lo0;
        mine[2 * q2 + 1] = c ? hi1 : lo1;
      }
      if (2 * i < p.M)
#pragma unroll
        for (int q2 = 0; q2 < HQ; ++q2) {
          const int jc = (n0 + c0) / 2 + (c ? HQ + q2 : q2);
          if (2 * jc < p.N) {
            // even lane: mine = (ReA ReB, ReA ImB), got = (ImA ReB, ImA ImB); odd lane the reverse
            const double rr = c ? got[2 * q2] : mine[2 * q2], ri = c ? got[2 * q2 + 1] : mine[2 * q2 + 1];
            const double ir = c ? mine[2 * q2] : got[2 * q2], ii = c ? mine[2 * q2 + 1] : got[2 * q2 + 1];
            zd x = zmk(rr - ii, ri + ir);
            zd* w = o + i * p.ldr + jc * p.ldc;
            if (p.osub > 0) { const zd g = *w; x = zmk(g.x - x.x, g.y - x.y); }
            else if (p.osub < 0) { const zd g = *w; x = zmk(g.x + x.x, g.y + x.y); }
            *w = x;
          }
        }
    } else {  // OZ_OUT_ROWS: real row 2 i + c -> complex row i; even lanes write the first HB/2 columns
      zd* o = (zd*)p.out + (size_t)b * p.sout;
      const int i = m >> 1, c = m & 1;
      double u[HB / 2], w2[HB / 2];
#pragma unroll
      for (int j = 0; j < HB / 2; ++j) {
        const double send = c ? v[j] : v[HB / 2 + j];  // odd lanes send their first half, even their second
        const double got = __shfl_xor_sync(0xffffffffu, send, 1);
        u[j] = c ? got : v[j];                         // real part of column (c ? HB/2 + j : j)
        w2[j] = c ? v[HB / 2 + j] : got;               // imaginary part
      }
      if (2 * i < p.M)
#pragma unroll
        for (int j = 0; j < HB / 2; ++j) {
          const int n = n0 + c0 + (c ? HB / 2 : 0) + j;
          if (n < p.N) {
            zd* w = o + i * p.ldr + n * p.ldc;
            zd x = zmk(u[j], w2[j]);
            if (p.osub) { const zd g = *w; x = zmk(g.x - x.x, g.y - x.y); }
            *w = x;
          }
        }
    }
  }
  oz_fence_before();
  if (tid == 0) *consumed_sh = 0;  // the next tile's chunk count (read by the producer on abort)
  __syncthreads();  // TMEM reads and the shared B blocks are free for the next tile
  if (*abort_flag || !done_ok) break;
  }  // tiles
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tbase), "r"(ncols) : "memory");
}

// ---------------------------------------------------------------------------------------
// Host helpers
// ---------------------------------------------------------------------------------------
typedef CUresult (*oz_encode_fn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                 const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                 CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

static inline oz_encode_fn oz_encoder() {
  static oz_encode_fn fn = nullptr;
  if (!fn) {
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = (oz_encode_fn)f;
  }
  return fn;
}

// 2-D map over a slice buffer [rows_total][Kpad] of BF16, box 64 x box_rows, 128-byte swizzle.
static inline int oz_tmap(CUtensorMap* m, void* base, int Kpad, long long rows_total, int box_rows) {
  oz_encode_fn enc = oz_encoder();
  if (!enc) return 1;
  const cuuint64_t dims[2] = {(cuuint64_t)Kpad, (cuuint64_t)rows_total};
  const cuuint64_t strides[1] = {(cuuint64_t)Kpad * 2};
  const cuuint32_t box[2] = {OZ_KC, (cuuint32_t)box_rows};
  const cuuint32_t es[2] = {1, 1};
  return enc(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, base, dims, strides, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE,
             CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) ==
                 CUDA_SUCCESS
             ? 0
             : 1;
}

// Digit width and count for a K extent: every diagonal partial sum stays an integer below
// 2^24 (S pairs at most, each below K (2^b - 1)^2), and S b >= OZ_TARGET_BITS.
static inline int oz_pick(int Kpad, int* bits, int* S) {
  for (int b = 7; b >= 4; --b) {
    const int s = (OZ_TARGET_BITS + b - 1) / b;
    const double bound = (double)s * Kpad * (double)((1 << b) - 1) * (double)((1 << b) - 1);
    if (bound < 16777216.0) { *bits = b; *S = s; return 0; }
  }
  return 1;
}

static inline int oz_round(int x, int m) { return (x + m - 1) / m * m; }

// Largest L such that sum_D |acc_D| 2^(L - b D) < 2^62 for any inputs (|acc_D| below
// min(2^24, pairs(D) K (2^b - 1)^2)): the combined integer keeps as many low bits as
// 64 bits allow.
static inline int oz_shift(int Kpad, int b, int S, int nd) {
  double z = 0.0;
  for (int D = 2; D < nd + 2; ++D) {
    const int pairs = std::min(D - 1, std::min(S, 2 * S + 1 - D));
    const double acc = std::min(16777216.0, (double)pairs * Kpad * (double)((1 << b) - 1) * ((1 << b) - 1));
    z += std::ldexp(acc, -b * D);
  }
  return (int)std::floor(62.0 - std::log2(z));
}

// Tile width and ring depth that fit 227 KB of shared memory; 1 when none does.  A CTA's
// time is dominated by the latency of streaming its A chunks, so a grid that does not fill
// the GPU (narrow = 1) takes BN = 16: half the resident B and twice the ring depth.
static inline int oz_pick_tile(int S, int nkc, int* bn, int* nst, int narrow = 0) {
  const size_t cap = 232448;
  const int w0 = narrow ? 16 : 32;
  for (int w = w0; w >= 16; w -= 16)
    for (int st = 8; st >= 2; --st)
      if (oz_smem_bytes(w, S, nkc, st) <= cap) { *bn = w; *nst = st; return 0; }
  return 1;
}
