// Device-side lattice-resolved observables: the predefined equal-time and time-displaced
// measurements that ham%Obser / ham%ObserT run with the Green functions of the sweep
// (Prog/Predefined_Obs_mod.F90:137-330 equal time: Green, SpinMz (SpinZ, SpinXY, SpinT), Den;
// :330-600 time displaced; N_FL = 1 models: Green, SpinSUN, Den), accumulated per chain as
// Obs_Latt(imj, nt, no_I, no_J), Obs_Latt0(no), the measurement count and the sign sum, the
// arrays Print_bin_Latt normalises (Prog/observables_mod.F90:355-500).
//
// A contribution of the site pair (i, j) goes to R = imj(cell(i), cell(j)) and the orbitals
// (orb(i), orb(j)).  One thread owns one output (R, no_I, no_J) and sums over the cells I,
// with J = jof(I, R) the cell at distance R from I, in a fixed order: no atomics, the same
// result for the same G.  Weights w = ZP ZS = Phase / Re(Phase) sign(Re(Phase)).
#pragma once
#include "common.cuh"

struct LattObsParams {
  int N, F, nsun, ncell, norb, nnames;
  int L1;                // time slices of the accumulator: 1 (equal time) or Ltrot + 1
  const int* site_of;    // [ncell][norb] site of (cell, orbital)
  const int* jof;        // [ncell][ncell] jof[I ncell + R]: the cell J with imj(I, J) = R
  const zd* phase;       // [chain]
  zd* acc;               // [chain][nnames][ncell][L1][norb][norb]
  zd* acc0;              // [chain][nnames][norb]
  double* cnt;           // [chain][2]: measurements, sum of ZS
};

ALF_DEV zd lobs_weight(zd ph, double* zs) {
  const double s = ph.x > 0.0 ? 1.0 : (ph.x < 0.0 ? -1.0 : 0.0);
  *zs = s;
  return zmk(ph.x / ph.x * s, ph.y / ph.x * s);  // (Phase / Re Phase) ZS
}

// Equal time, G = [chain][F][N][N] column-major in the callback's frame.
// grid (ceil(ncell norb^2 / 128), chains), 128 threads.
__global__ void k_obs_latt_eq(const zd* G, LattObsParams p) {
  const int c = blockIdx.y, no = p.norb;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const long long NN = (long long)p.N * p.N;
  const zd* G0 = G + (long long)c * p.F * NN;
  const zd* G1 = G0 + (p.F == 2 ? NN : 0);
  double zs;
  const zd w = lobs_weight(p.phase[c], &zs);
  const double ns = (double)p.nsun;
  const int nout = p.ncell * no * no;
  zd* acc = p.acc + (long long)c * p.nnames * nout;
  if (t < nout) {
    const int R = t / (no * no), oi = (t / no) % no, oj = t % no;
    zd s[5] = {zmk(0, 0), zmk(0, 0), zmk(0, 0), zmk(0, 0), zmk(0, 0)};
    for (int I = 0; I < p.ncell; ++I) {
      const int i = p.site_of[I * no + oi], J = p.jof[I * p.ncell + R], j = p.site_of[J * no + oj];
      const double dij = (i == j) ? 1.0 : 0.0;
      const zd g0 = G0[i + (long long)j * p.N], c0 = zsub(zmk(dij, 0.0), G0[j + (long long)i * p.N]);
      const zd ci0 = zsub(zmk(1.0, 0.0), G0[i + (long long)i * p.N]);
      const zd cj0 = zsub(zmk(1.0, 0.0), G0[j + (long long)j * p.N]);
      if (p.F == 1) {  // Green, SpinSUN, Den
        const zd cg = zmul(c0, g0);
        s[0] = zadd(s[0], zscale(c0, ns));
        s[1] = zadd(s[1], zscale(cg, ns));
        s[2] = zadd(s[2], zadd(zscale(zmul(ci0, cj0), ns * ns), zscale(cg, ns)));
        continue;
      }
      const zd g1 = G1[i + (long long)j * p.N], c1 = zsub(zmk(dij, 0.0), G1[j + (long long)i * p.N]);
      const zd ci1 = zsub(zmk(1.0, 0.0), G1[i + (long long)i * p.N]);
      const zd cj1 = zsub(zmk(1.0, 0.0), G1[j + (long long)j * p.N]);
      s[0] = zadd(s[0], zscale(zadd(c0, c1), ns));                 // Green
      const zd same = zadd(zmul(c0, g0), zmul(c1, g1));
      if (p.nsun == 1) {
        const zd dzi = zsub(ci1, ci0), dzj = zsub(cj1, cj0);
        const zd zz = zadd(same, zmul(dzi, dzj));
        const zd zxy = zadd(zmul(c0, g1), zmul(c1, g0));
        s[1] = zadd(s[1], zz);                                    // SpinZ
        s[2] = zadd(s[2], zxy);                                   // SpinXY
        s[3] = zadd(s[3], zscale(zadd(zscale(zxy, 2.0), zz), 1.0 / 3.0));  // SpinT
      }
      const zd zi = zscale(zadd(ci0, ci1), ns), zj = zscale(zadd(cj0, cj1), ns);
      s[4] = zadd(s[4], zadd(zmul(zi, zj), zscale(same, ns)));     // Den
    }
    for (int k = 0; k < p.nnames; ++k) {
      zd* a = acc + (long long)k * nout + t;  // L1 = 1
      *a = zadd(*a, zmul(s[k], w));
    }
  }
  if (t < no) {  // Obs_Latt0 of orbital t: sum over the cells
    zd dz = zmk(0, 0), zi = zmk(0, 0);
    for (int I = 0; I < p.ncell; ++I) {
      const int i = p.site_of[I * no + t];
      const zd ci0 = zsub(zmk(1.0, 0.0), G0[i + (long long)i * p.N]);
      if (p.F == 1) { zi = zadd(zi, zscale(ci0, ns)); continue; }
      const zd ci1 = zsub(zmk(1.0, 0.0), G1[i + (long long)i * p.N]);
      dz = zadd(dz, zsub(ci1, ci0));
      zi = zadd(zi, zscale(zadd(ci0, ci1), ns));
    }
    zd* a0 = p.acc0 + (long long)c * p.nnames * no;
    if (p.F == 1) {
      a0[2 * no + t] = zadd(a0[2 * no + t], zmul(zi, w));
    } else {
      if (p.nsun == 1) {
        a0[1 * no + t] = zadd(a0[1 * no + t], zmul(dz, w));
        a0[3 * no + t] = zadd(a0[3 * no + t], zmul(zscale(dz, 0.57735026918962576451), w));  // 1/sqrt(3)
      }
      a0[4 * no + t] = zadd(a0[4 * no + t], zmul(zi, w));
    }
  }
  if (t == 0) {
    p.cnt[2 * c] += 1.0;
    p.cnt[2 * c + 1] += zs;
  }
}

// Time displaced at slice nt, Q = [chain][4][F][N][N] = [GT0, G0T, G00, GTT].
// grid (ceil(ncell norb^2 / 128), chains), 128 threads.
__global__ void k_obs_latt_tau(const zd* Q, int nt, LattObsParams p) {
  const int c = blockIdx.y, no = p.norb, F = p.F;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const long long NN = (long long)p.N * p.N;
  const zd* q = Q + (long long)c * 4 * F * NN;
  const zd *GT0 = q, *G0T = q + F * NN, *G00 = q + 2 * F * NN, *GTT = q + 3 * F * NN;
  double zs;
  const zd w = lobs_weight(p.phase[c], &zs);
  const double ns = (double)p.nsun;
  const int nout = p.ncell * no * no;
  const long long per_name = (long long)p.ncell * p.L1 * no * no;
  zd* acc = p.acc + (long long)c * p.nnames * per_name;
  auto at = [&](const zd* X, int f, int i, int j) { return X[f * NN + i + (long long)j * p.N]; };
  if (t < nout) {
    const int R = t / (no * no), oi = (t / no) % no, oj = t % no;
    zd s[5] = {zmk(0, 0), zmk(0, 0), zmk(0, 0), zmk(0, 0), zmk(0, 0)};
    for (int I = 0; I < p.ncell; ++I) {
      const int i = p.site_of[I * no + oi], J = p.jof[I * p.ncell + R], j = p.site_of[J * no + oj];
      if (F == 1) {  // Green, SpinSUN, Den
        const zd gt0 = at(GT0, 0, i, j), conn = zmul(at(G0T, 0, j, i), gt0);
        const zd zi = zscale(zsub(zmk(1.0, 0.0), at(GTT, 0, i, i)), ns);
        const zd zj = zscale(zsub(zmk(1.0, 0.0), at(G00, 0, j, j)), ns);
        s[0] = zadd(s[0], gt0);
        s[1] = zsub(s[1], zscale(conn, ns));
        s[2] = zadd(s[2], zsub(zmul(zi, zj), zscale(conn, ns)));
        continue;
      }
      const zd a0 = at(GT0, 0, i, j), a1 = at(GT0, 1, i, j);
      const zd b0 = at(G0T, 0, j, i), b1 = at(G0T, 1, j, i);
      s[0] = zadd(s[0], zscale(zadd(a0, a1), 0.5));
      const zd dtt = zsub(at(GTT, 0, i, i), at(GTT, 1, i, i));
      const zd d00 = zsub(at(G00, 0, j, j), at(G00, 1, j, j));
      const zd same = zadd(zmul(b0, a0), zmul(b1, a1));
      const zd zz = zsub(zmul(dtt, d00), same);
      const zd zxy = zneg(zadd(zmul(b0, a1), zmul(b1, a0)));
      s[1] = zadd(s[1], zz);
      s[2] = zadd(s[2], zxy);
      s[3] = zadd(s[3], zscale(zadd(zscale(zxy, 2.0), zz), 1.0 / 3.0));
      const zd zi = zscale(zadd(zsub(zmk(1.0, 0.0), at(GTT, 0, i, i)), zsub(zmk(1.0, 0.0), at(GTT, 1, i, i))), ns);
      const zd zj = zscale(zadd(zsub(zmk(1.0, 0.0), at(G00, 0, j, j)), zsub(zmk(1.0, 0.0), at(G00, 1, j, j))), ns);
      s[4] = zadd(s[4], zsub(zmul(zi, zj), zscale(same, ns)));
    }
    for (int k = 0; k < p.nnames; ++k) {
      zd* a = acc + (long long)k * per_name + ((long long)R * p.L1 + nt) * no * no + oi * no + oj;
      *a = zadd(*a, zmul(s[k], w));
    }
  }
  if (t < no) {
    zd dtt = zmk(0, 0), zi = zmk(0, 0);
    for (int I = 0; I < p.ncell; ++I) {
      const int i = p.site_of[I * no + t];
      if (F == 1) { zi = zadd(zi, zscale(zsub(zmk(1.0, 0.0), at(GTT, 0, i, i)), ns)); continue; }
      dtt = zadd(dtt, zsub(at(GTT, 0, i, i), at(GTT, 1, i, i)));
      zi = zadd(zi, zscale(zadd(zsub(zmk(1.0, 0.0), at(GTT, 0, i, i)), zsub(zmk(1.0, 0.0), at(GTT, 1, i, i))), ns));
    }
    zd* a0 = p.acc0 + (long long)c * p.nnames * no;
    if (F == 1) {
      a0[2 * no + t] = zadd(a0[2 * no + t], zmul(zi, w));
    } else {
      a0[1 * no + t] = zsub(a0[1 * no + t], zmul(dtt, w));
      a0[3 * no + t] = zsub(a0[3 * no + t], zmul(zscale(dtt, 0.57735026918962576451), w));
      a0[4 * no + t] = zadd(a0[4 * no + t], zmul(zi, w));
    }
  }
  if (t == 0 && nt == 0) {
    p.cnt[2 * c] += 1.0;
    p.cnt[2 * c + 1] += zs;
  }
}
