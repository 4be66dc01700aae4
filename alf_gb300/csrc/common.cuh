// Shared device helpers for the alfgpu kernels (sm_103a).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/alfgpu.h"

typedef double2 zd;  // complex128, (x = re, y = im)

#define ALF_DEV __device__ __forceinline__
#define ALF_HD __host__ __device__ __forceinline__

ALF_HD zd zmk(double r, double i) { zd z; z.x = r; z.y = i; return z; }
ALF_HD zd zadd(zd a, zd b) { return zmk(a.x + b.x, a.y + b.y); }
ALF_HD zd zsub(zd a, zd b) { return zmk(a.x - b.x, a.y - b.y); }
ALF_HD zd zmul(zd a, zd b) { return zmk(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x); }
ALF_HD zd zconj(zd a) { return zmk(a.x, -a.y); }
// c + a b and c - a b as two FMA chains (four FP64 instructions; zadd(c, zmul(a, b)) takes a
// multiply, an FMA and an add per component)
ALF_HD zd zfma(zd a, zd b, zd c) { return zmk(fma(a.x, b.x, fma(-a.y, b.y, c.x)), fma(a.x, b.y, fma(a.y, b.x, c.y))); }
ALF_HD zd zfms(zd a, zd b, zd c) {
  return zmk(fma(-a.x, b.x, fma(a.y, b.y, c.x)), fma(-a.x, b.y, fma(-a.y, b.x, c.y)));
}
ALF_HD zd zscale(zd a, double s) { return zmk(a.x * s, a.y * s); }
ALF_HD double zabs(zd a) { return hypot(a.x, a.y); }
ALF_HD zd zneg(zd a) { return zmk(-a.x, -a.y); }
// Smith's complex division (robust against overflow).
ALF_HD zd zdiv(zd a, zd b) {
  if (fabs(b.x) >= fabs(b.y)) {
    double r = b.y / b.x, d = b.x + b.y * r;
    return zmk((a.x + a.y * r) / d, (a.y - a.x * r) / d);
  } else {
    double r = b.x / b.y, d = b.y + b.x * r;
    return zmk((a.x * r + a.y) / d, (a.y * r - a.x) / d);
  }
}
ALF_HD zd zexp(zd a) {
  double e = exp(a.x);
  double s, c;
  sincos(a.y, &s, &c);
  return zmk(e * c, e * s);
}
ALF_HD zd zinv(zd a) { return zdiv(zmk(1.0, 0.0), a); }

// ---------------------------------------------------------------------------
// Thread-block cluster helpers (inline PTX; barrier.cluster has release/acquire
// semantics at cluster scope, which orders global and shared memory).
// ---------------------------------------------------------------------------
ALF_DEV unsigned cluster_ctarank() {
  unsigned r;
  asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
  return r;
}
ALF_DEV unsigned cluster_nctarank() {
  unsigned r;
  asm volatile("mov.u32 %0, %%cluster_nctarank;" : "=r"(r));
  return r;
}
ALF_DEV void cluster_sync() {
  asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
}
// Address of `p` (a shared-memory variable of this CTA) in the shared window of CTA `rank`.
ALF_DEV uint32_t dsmem_addr(const void* p, unsigned rank) {
  uint32_t a = (uint32_t)__cvta_generic_to_shared(p), r;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(a), "r"(rank));
  return r;
}
ALF_DEV double dsmem_ld_f64(uint32_t addr) {
  double v;
  asm volatile("ld.shared::cluster.f64 %0, [%1];" : "=d"(v) : "r"(addr) : "memory");
  return v;
}
ALF_DEV int dsmem_ld_s32(uint32_t addr) {
  int v;
  asm volatile("ld.shared::cluster.s32 %0, [%1];" : "=r"(v) : "r"(addr) : "memory");
  return v;
}

// Warp reductions
ALF_DEV double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
ALF_DEV double warp_max(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}
ALF_DEV zd warp_zsum(zd v) { return zmk(warp_sum(v.x), warp_sum(v.y)); }

// Counter-based uniform stream shared with the oracle's harness:
// u = (splitmix64(key(seed, chain) + (counter+1)*golden) >> 11) * 2^-53.
ALF_HD uint64_t alf_mix64(uint64_t z) {
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
ALF_HD uint64_t alf_chain_key(uint64_t seed, uint64_t chain) {
  return alf_mix64((seed ^ (chain * 0xD1B54A32D192ED03ull)) + 0x9E3779B97F4A7C15ull);
}
ALF_HD double alf_uniform(uint64_t key, uint64_t counter) {
  uint64_t z = alf_mix64(key + (counter + 1ull) * 0x9E3779B97F4A7C15ull);
  return (double)(z >> 11) * (1.0 / 9007199254740992.0);
}

// Type-2 field tables (Prog/Fields_mod.F90:270-301); index s+2.
struct FieldTables {
  double phi[2][5];   // [type-1][s+2]
  double gama[2][5];
  double grat[2][5][5];  // [type-1][s_old+2][s_new+2] = gama(s_new) / gama(s_old)
  int8_t flip[5][3];  // type 2
};
