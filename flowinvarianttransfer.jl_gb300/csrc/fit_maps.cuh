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
  bool keep = true;
#pragma unroll
  for (int d = 0; d < 3; ++d) {   // unrolled: k stays in registers
    if (d < g.nd) {
      const int N = g.N[d];
      const int a = (k[d] <= N / 2) ? k[d] : N - k[d];
      keep = keep && a < N / 3;
    }
  }
  return keep;
}

FIT_D void decode_half(const GridDesc& g, long i, int* g0, int* g1, int* g2) {
  if (g.Mhalf <= 0x7fffffffL) {   // 32-bit index arithmetic (every grid up to 1024^3 fits)
    const unsigned u = (unsigned)i, m0 = (unsigned)g.Mh0, m1 = (unsigned)g.M[1];
    const unsigned r = u / m0;
    const unsigned q = r / m1;
    *g0 = (int)(u - r * m0);
    *g1 = (int)(r - q * m1);
    *g2 = (int)q;
    return;
  }
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

// CT: arithmetic type (float for single-precision data, double otherwise).
template <typename CT>
FIT_D typename Vec2<CT>::t ld_ct(const void* p, int f64, long i) {
  typename Vec2<CT>::t r;
  if (f64) {
    const double2 v = reinterpret_cast<const double2*>(p)[i];
    r.x = (CT)v.x;
    r.y = (CT)v.y;
  } else {
    const float2 v = reinterpret_cast<const float2*>(p)[i];
    r.x = (CT)v.x;
    r.y = (CT)v.y;
  }
  return r;
}

template <typename CT>
FIT_D void carrier_at_t(const GridDesc& g, const KTab& kt, const void* car, int f64, long cs, int nc, int inv,
                        long lin, const int* k, typename Vec2<CT>::t* C) {
  typedef typename Vec2<CT>::t C2;
  C2 u[3];
#pragma unroll
  for (int c = 0; c < 3; ++c) u[c] = c < nc ? ld_ct<CT>(car, f64, lin + cs * c) : mkc<C2>(0, 0);
  if (inv == INV_KE || inv == INV_SCALAR) {
#pragma unroll
    for (int c = 0; c < 3; ++c)
      if (c < nc) C[c] = u[c];
    return;
  }
  const CT kx = ktab_at<CT>(kt, 0, k[0]);
  const CT ky = g.nd >= 2 ? ktab_at<CT>(kt, 1, k[1]) : (CT)0;
  const CT kz = g.nd >= 3 ? ktab_at<CT>(kt, 2, k[2]) : (CT)0;
  if (inv == INV_ENSTROPHY && g.nd == 2) {
    // w = i (kx uy - ky ux)
    const C2 w = mkc<C2>(-(kx * u[1].y - ky * u[0].y), kx * u[1].x - ky * u[0].x);
    C[0] = mkc<C2>(-w.y * ky, w.x * ky);
    C[1] = mkc<C2>(w.y * kx, -w.x * kx);
    return;
  }
  // curl: i (k x u)
  C2 w[3];
  w[0] = mkc<C2>(-(ky * u[2].y - kz * u[1].y), ky * u[2].x - kz * u[1].x);
  w[1] = mkc<C2>(-(kz * u[0].y - kx * u[2].y), kz * u[0].x - kx * u[2].x);
  w[2] = mkc<C2>(-(kx * u[1].y - ky * u[0].y), kx * u[1].x - ky * u[0].x);
  if (inv == INV_HELICITY) {
    C[0] = w[0]; C[1] = w[1]; C[2] = w[2];
    return;
  }
  C[0] = mkc<C2>(-(ky * w[2].y - kz * w[1].y), ky * w[2].x - kz * w[1].x);
  C[1] = mkc<C2>(-(kz * w[0].y - kx * w[2].y), kz * w[0].x - kx * w[2].x);
  C[2] = mkc<C2>(-(kx * w[1].y - ky * w[0].y), kx * w[1].x - ky * w[0].x);
}

FIT_D void carrier_at(const GridDesc& g, const KTab& kt, const void* car, int f64, long cs, int nc, int inv,
                      long lin, const int* k, double2* C) {
  carrier_at_t<double>(g, kt, car, f64, cs, nc, inv, lin, k, C);
}

// N-grid linear index -> per-axis indices (32-bit arithmetic when the grid allows it).
FIT_D void decode_full(const GridDesc& g, long i, int* k) {
  if (g.Ntot <= 0x7fffffffL) {
    const unsigned u = (unsigned)i, n0 = (unsigned)g.N[0], n1 = (unsigned)g.N[1];
    const unsigned r = u / n0;
    const unsigned q = r / n1;
    k[0] = (int)(u - r * n0);
    k[1] = (int)(r - q * n1);
    k[2] = (int)q;
    return;
  }
  k[0] = (int)(i % g.N[0]);
  const long r = i / g.N[0];
  k[1] = (int)(r % g.N[1]);
  k[2] = (int)(r / g.N[1]);
}

}  // namespace fit
