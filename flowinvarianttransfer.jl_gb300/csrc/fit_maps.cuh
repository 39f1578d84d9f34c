// Device-side index maps between the transform grid and the data grid, the 2/3 predicate, and
// the effective carriers of the transfer densities (shared by the generic and fused paths).
#pragma once

#include "fit_ops.cuh"

namespace fit {

// ---- index helpers ---------------------------------------------------------------------------

struct KIdx {
  long lin;   // linear N-grid index, -1 = absent
  int k[3];   // per-axis N-grid index
};

FIT_D bool in_fset(int f, int N) { return f >= -(N / 2) && f <= (N + 1) / 2 - 1; }
FIT_D int fmod_pos(int f, int N) { int r = f % N; return r < 0 ? r + N : r; }

// N-grid mode at signed transform-grid frequency (f0,f1,f2) of the padded map.
FIT_D KIdx kidx_of_freq(const GridDesc& g, int f0, int f1, int f2) {
  KIdx r;
  r.lin = -1;
  r.k[0] = r.k[1] = r.k[2] = 0;
  const int f[3] = {f0, f1, f2};
  long lin = 0, stride = 1;
  for (int d = 0; d < 3; ++d) {
    if (!in_fset(f[d], g.N[d])) return r;
    r.k[d] = fmod_pos(f[d], g.N[d]);
    lin += r.k[d] * stride;
    stride *= g.N[d];
  }
  r.lin = lin;
  return r;
}

FIT_D int signed_freq(int i, int M) { return (2 * i <= M) ? i : i - M; }

// Both N-grid modes feeding half-spectrum mode g: kA at +g, kB at -g.
FIT_D void map_pair(const GridDesc& g, int g0, int g1, int g2, KIdx* kA, KIdx* kB) {
  if (!g.padded) {
    kA->k[0] = g0; kA->k[1] = g1; kA->k[2] = g2;
    kA->lin = g0 + (long)g.N[0] * (g1 + (long)g.N[1] * g2);
    kB->k[0] = (g.N[0] - g0) % g.N[0];
    kB->k[1] = (g.N[1] - g1) % g.N[1];
    kB->k[2] = (g.N[2] - g2) % g.N[2];
    kB->lin = kB->k[0] + (long)g.N[0] * (kB->k[1] + (long)g.N[1] * kB->k[2]);
    return;
  }
  const int f0 = g0, f1 = signed_freq(g1, g.M[1]), f2 = signed_freq(g2, g.M[2]);
  *kA = kidx_of_freq(g, f0, f1, f2);
  *kB = kidx_of_freq(g, -f0, -f1, -f2);
}

// Orszag 2/3 keep predicate on the N grid (src/NonlinearTerm.jl:134-141): every axis index
// magnitude below N_d div 3.
FIT_D bool keep23(const GridDesc& g, const int* k) {
  for (int d = 0; d < g.nd; ++d) {
    const int N = g.N[d];
    const int a = (k[d] <= N / 2) ? k[d] : N - k[d];
    if (a >= N / 3) return false;
  }
  return true;
}

FIT_D void decode_half(const GridDesc& g, long i, int* g0, int* g1, int* g2) {
  *g0 = (int)(i % g.Mh0);
  const long r = i / g.Mh0;
  *g1 = (int)(r % g.M[1]);
  *g2 = (int)(r / g.M[1]);
}

FIT_D double2 ld_c(const void* p, int f64, long i) {
  if (f64) return reinterpret_cast<const double2*>(p)[i];
  const float2 v = reinterpret_cast<const float2*>(p)[i];
  return make_double2((double)v.x, (double)v.y);
}

template <typename V>
FIT_D V to_v(double2 a);
template <>
FIT_D float2 to_v<float2>(double2 a) { return make_float2((float)a.x, (float)a.y); }
template <>
FIT_D double2 to_v<double2>(double2 a) { return a; }

FIT_D double2 dmul_i(double2 a, double k) { return make_double2(-a.y * k, a.x * k); }   // i*k*a

// ---- effective carriers ------------------------------------------------------------------------
// Every transfer density of src/Invariants.jl:40-104 is linear in N, t = sum_c Re(conj(C_c) N_c):
//   KE / passive scalar: C = u;   helicity: C = i k x u;
//   enstrophy 2D: w = i(kx uy - ky ux), C = (w * i ky, -w * i kx);   enstrophy 3D: C = ik x (ik x u).

FIT_D void carrier_at(const GridDesc& g, const KTab& kt, const void* car, int f64, long cs, int nc, int inv,
                      long lin, const int* k, double2* C) {
  double2 u[3];
  for (int c = 0; c < nc && c < 3; ++c) u[c] = ld_c(car, f64, lin + cs * c);
  if (inv == INV_KE || inv == INV_SCALAR) {
    for (int c = 0; c < nc; ++c) C[c] = u[c];
    return;
  }
  const double kx = kt.k[0][k[0]];
  const double ky = g.nd >= 2 ? kt.k[1][k[1]] : 0.0;
  const double kz = g.nd >= 3 ? kt.k[2][k[2]] : 0.0;
  if (inv == INV_ENSTROPHY && g.nd == 2) {
    // w = i (kx uy - ky ux)
    const double2 w = make_double2(-(kx * u[1].y - ky * u[0].y), kx * u[1].x - ky * u[0].x);
    C[0] = dmul_i(w, ky);
    C[1] = dmul_i(w, -kx);
    return;
  }
  // curl: i (k x u)
  double2 w[3];
  w[0] = make_double2(-(ky * u[2].y - kz * u[1].y), ky * u[2].x - kz * u[1].x);
  w[1] = make_double2(-(kz * u[0].y - kx * u[2].y), kz * u[0].x - kx * u[2].x);
  w[2] = make_double2(-(kx * u[1].y - ky * u[0].y), kx * u[1].x - ky * u[0].x);
  if (inv == INV_HELICITY) {
    C[0] = w[0]; C[1] = w[1]; C[2] = w[2];
    return;
  }
  C[0] = make_double2(-(ky * w[2].y - kz * w[1].y), ky * w[2].x - kz * w[1].x);
  C[1] = make_double2(-(kz * w[0].y - kx * w[2].y), kz * w[0].x - kx * w[2].x);
  C[2] = make_double2(-(kx * w[1].y - ky * w[0].y), kx * w[1].x - ky * w[0].x);
}


}  // namespace fit
