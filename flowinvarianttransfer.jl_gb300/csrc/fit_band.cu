// Smooth band-to-band transfer T(K,Q) (src/BandTransfer.jl:24-113, Eyink & Aluie 2009).
//
// Bands are a partition of unity of log-Gaussian weights w_n(kappa) over the shell coordinate
// kappa (src/BandTransfer.jl:24-46). For each band m the advected field is w_m * f, its nonlinear
// term N̂_m (advected by the full velocity) is formed exactly as for a shell-to-shell mediator,
// and T(n, m) = sum_k w_n(k) t_m(k) with t_m the invariant's transfer density of N̂_m against the
// full field. The weights live on the transform grid's half spectrum (both conjugate modes of a
// half mode share |k|): one table feeds the gather (w_m * f) and the weighted binning.
#include <math.h>
#include <string.h>

#include <vector>

#include "fit_gb300.h"
#include "fit_maps.cuh"
#include "fit_plan.cuh"

namespace fit {

// Shell coordinate of N-grid mode k over the dims mask (src/ShellBinning.jl:19-36): sum of k_d^2 in
// increasing d, every operation rounded, in FP64 or in Float32 when the wavenumbers are Float32.
FIT_D double band_kappa(const GridDesc& g, const KTab& kt, unsigned dims, int f32, const int* k) {
  if (f32) {
    float s = 0.f;
    for (int d = 0; d < g.nd; ++d)
      if (dims & (1u << d)) {
        const float kd = (float)kt.k[d][k[d]];
        s = __fadd_rn(s, __fmul_rn(kd, kd));
      }
    return (double)__fsqrt_rn(s);
  }
  double s = 0.0;
  for (int d = 0; d < g.nd; ++d)
    if (dims & (1u << d)) {
      const double kd = kt.k[d][k[d]];
      s = __dadd_rn(s, __dmul_rn(kd, kd));
    }
  return __dsqrt_rn(s);
}

// Normalised weights of transform-grid half mode (g0, g1, g2) (zero when no N-grid mode maps to it):
// w_n = exp(-ln(kappa / c_n)^2 / (2 logwidth^2)) / sum over bands, 0 at kappa = 0
// (src/BandTransfer.jl:24-48).
FIT_D void band_weights_at(const GridDesc& g, const KTab& kt, unsigned dims, int f32, const double* centers, int nb,
                           double logwidth, int g0, int g1, int g2, double* wn) {
  KIdx kA, kB;
  map_pair(g, g0, g1, g2, &kA, &kB);
  const KIdx& k = kA.lin >= 0 ? kA : kB;
  double kappa = 0.0;
  if (k.lin >= 0) kappa = band_kappa(g, kt, dims, f32, k.k);
  double sum = 0.0;
#pragma unroll
  for (int n = 0; n < 16; ++n) {
    wn[n] = 0.0;
    if (n < nb && kappa > 0.0) {
      const double r = log(kappa / centers[n]);
      wn[n] = exp(-(r * r) / (2.0 * logwidth * logwidth));
      sum += wn[n];
    }
  }
#pragma unroll
  for (int n = 0; n < 16; ++n) wn[n] = sum > 0.0 ? wn[n] / sum : 0.0;
}

// w[n][i] for every half mode i of the transform grid.
template <typename S>
__global__ void k_band_weights(GridDesc g, KTab kt, unsigned dims, int f32, const double* __restrict__ centers,
                               int nb, double logwidth, S* __restrict__ w) {
  const long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (i >= g.Mhalf) return;
  int g0, g1, g2;
  decode_half(g, i, &g0, &g1, &g2);
  double wn[16];
  band_weights_at(g, kt, dims, f32, centers, nb, logwidth, g0, g1, g2, wn);
#pragma unroll
  for (int n = 0; n < 16; ++n)
    if (n < nb) w[(long)n * g.Mhalf + i] = (S)wn[n];
}

// The same weights on the live box of the fused FP32 path only, layout [n][kz'][kx + KX ky'] (box mode
// (kx, ky' - K, kz' - K)): a quarter of the half spectrum at 512^3 with the 2/3 rule.
__global__ void k_band_weights_box(GridDesc g, KTab kt, int K, int KX, int KY, unsigned dims, int f32,
                                   const double* __restrict__ centers, int nb, double logwidth, float* __restrict__ w) {
  const long P1 = (long)KX * KY, BL = P1 * KY;
  const long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (i >= BL) return;
  const long col = i % P1;
  const int kz = (int)(i / P1), kx = (int)(col % KX), ky = (int)(col / KX);
  double wn[16];
  band_weights_at(g, kt, dims, f32, centers, nb, logwidth, kx, fmod_pos(ky - K, g.M[1]), fmod_pos(kz - K, g.M[2]),
                  wn);
#pragma unroll
  for (int n = 0; n < 16; ++n)
    if (n < nb) w[(long)n * BL + i] = (float)wn[n];
}

// out[n] = sum over half modes i with seff(i) != 0 of w[n][i] * sum_c Re(conj(ceff_c(i)) nh_c(i)).
// Per-thread sums in FP32 (single precision) are flushed to FP64 every 32 modes; FP64 data is
// accumulated in FP64 throughout.
template <typename V, typename CT, typename S>
__global__ void __launch_bounds__(256) k_band_bin(const V* __restrict__ nh, const V* __restrict__ ceff, int nc,
                                                  const uint16_t* __restrict__ seff, const S* __restrict__ w, int nb,
                                                  long Mhalf, double* __restrict__ partial) {
  double acc[16];
  CT part[16];
#pragma unroll
  for (int n = 0; n < 16; ++n) {
    acc[n] = 0.0;
    part[n] = 0;
  }
  const long step = (long)gridDim.x * blockDim.x;
  int cnt = 0;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < Mhalf; i += step) {
    if (seff[i]) {
      CT d = 0;
#pragma unroll
      for (int c = 0; c < 3; ++c)
        if (c < nc) {
          const V cf = ceff[(long)c * Mhalf + i];
          const V x = nh[(long)c * Mhalf + i];
          d += (CT)cf.x * (CT)x.x + (CT)cf.y * (CT)x.y;
        }
#pragma unroll
      for (int n = 0; n < 16; ++n)
        if (n < nb) part[n] += (CT)w[(long)n * Mhalf + i] * d;
    }
    if (++cnt == 32) {
      cnt = 0;
#pragma unroll
      for (int n = 0; n < 16; ++n) {
        acc[n] += (double)part[n];
        part[n] = 0;
      }
    }
  }
  __shared__ double red[8][16];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int n = 0; n < 16; ++n) {
    double v = acc[n] + (double)part[n];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if (lane == 0) red[warp][n] = v;
  }
  __syncthreads();
  if (threadIdx.x < nb) {
    double s = 0.0;
    for (int q = 0; q < (int)(blockDim.x >> 5); ++q) s += red[q][threadIdx.x];
    partial[(long)blockIdx.x * nb + threadIdx.x] = s;
  }
}

__global__ void k_band_reduce(const double* __restrict__ partial, int nblocks, int nb, double* __restrict__ out) {
  const int n = threadIdx.x;
  if (n >= nb) return;
  double s = 0.0;
  for (int b = 0; b < nblocks; ++b) s += partial[(long)b * nb + n];
  out[n] = s;
}

template <typename T>
static int band_run(fit_plan* p, const void* ud, const void* ad, int nb, int invariant, double* Td) {
  typedef typename Vec2<T>::t V;
  const GridDesc& g = p->g;
  FIT_TRY(carrier_and_bin_setup<T>(p, ud, invariant));
  const int nblocks = 2 * 152;
  FIT_TRY(ensure(p, &p->partial, sizeof(double) * nblocks * nb));
  for (int m = 0; m < nb; ++m) {
    FIT_TRY(nonlinear_half<T>(p, ud, ad, 0, m > 0, m + 1));
    if (sizeof(T) == 4)
      k_band_bin<V, float, T><<<nblocks, 256, 0, p->stream>>>((const V*)p->nh.p, (const V*)p->ceff.p, p->M,
                                                             (const uint16_t*)p->seff.p, (const T*)p->wtab.p, nb,
                                                             g.Mhalf, (double*)p->partial.p);
    else
      k_band_bin<V, double, T><<<nblocks, 256, 0, p->stream>>>((const V*)p->nh.p, (const V*)p->ceff.p, p->M,
                                                              (const uint16_t*)p->seff.p, (const T*)p->wtab.p, nb,
                                                              g.Mhalf, (double*)p->partial.p);
    FIT_LAUNCH_CHECK();
    k_band_reduce<<<1, 32, 0, p->stream>>>((const double*)p->partial.p, nblocks, nb, Td + (long)m * nb);
    FIT_LAUNCH_CHECK();
  }
  return FIT_OK;
}

}  // namespace fit

using namespace fit;

extern "C" int fit_band_to_band(fit_plan* p, const void* u_hat, const void* adv_hat, const double* centers,
                                int n_bands, double logwidth, uint32_t dims_mask, int coord_f32, int invariant,
                                double* T_colmajor, double* net, double* max_asym, int ptr_kind) {
  if (!p || !u_hat || !centers || !T_colmajor) {
    fit_set_error("NULL argument");
    return FIT_ERR_ARG;
  }
  if (n_bands < 1 || n_bands > 16) {
    fit_set_error("band-to-band transfer supports 1..16 bands (got %d)", n_bands);
    return FIT_ERR_ARG;
  }
  for (int n = 0; n < n_bands; ++n)
    if (!(centers[n] > 0.0) || (n > 0 && !(centers[n] > centers[n - 1]))) {
      fit_set_error("band centers must be positive and increasing");
      return FIT_ERR_ARG;
    }
  if (!(logwidth > 0.0)) {
    fit_set_error("logwidth must be positive");
    return FIT_ERR_ARG;
  }
  if (invariant < 0 || invariant > 3) {
    fit_set_error("unknown invariant %d", invariant);
    return FIT_ERR_ARG;
  }
  if (invariant == INV_HELICITY && !(p->nd == 3 && p->M == 3)) {
    fit_set_error("Helicity transfer is defined in 3D only (got nd=%d).", p->nd);
    return FIT_ERR_ARG;
  }
  if (!adv_hat && p->M < p->nd) {
    fit_set_error("self-advection needs >= nd components (pass advecting_hat)");
    return FIT_ERR_ARG;
  }
  const size_t cb = (p->io_f64 ? 16 : 8) * (size_t)p->g.Ntot;
  const void* ud = u_hat;
  const void* ad = adv_hat;
  if (ptr_kind != FIT_PTR_DEVICE) {
    FIT_TRY(ensure(p, &p->in_u, cb * p->M));
    FIT_CUDA_CHECK(cudaMemcpyAsync(p->in_u.p, u_hat, cb * p->M, cudaMemcpyHostToDevice, p->stream));
    ud = p->in_u.p;
    if (adv_hat) {
      FIT_TRY(ensure(p, &p->in_a, cb * p->Dadv));
      FIT_CUDA_CHECK(cudaMemcpyAsync(p->in_a.p, adv_hat, cb * p->Dadv, cudaMemcpyHostToDevice, p->stream));
      ad = p->in_a.p;
    }
  }
  if (!ad) ad = ud;
  // presence mask: one shell [0, inf) over the same coordinate (seff = 0 only for absent or
  // 2/3-discarded modes)
  const double all[2] = {0.0, 1e300};
  FIT_TRY(ensure_shells(p, all, 2, dims_mask, coord_f32));
  // weight table, cached per (centers, logwidth, dims, coordinate type, layout): on the live box for
  // FP32 cubic 3D plans of a fused size, else on the transform grid's half spectrum
  const bool box = p->prec == 32 && fz_box_ok(p);
  int bK = 0, bKX = 0, bKY = 0;
  long bP1 = 0;
  if (box) fz_box_geom(p, &bK, &bKX, &bKY, &bP1);
  const long nw = box ? bP1 * bKY : p->g.Mhalf;
  std::vector<double> key(centers, centers + n_bands);
  key.push_back(logwidth);
  key.push_back((double)dims_mask);
  key.push_back((double)coord_f32);
  key.push_back((double)p->prec);
  key.push_back((double)box);
  if (key != p->wtab_key) {
    const size_t wb = ((p->prec == 64 ? 8 : 4) * (size_t)n_bands * nw + 255) / 256 * 256;
    FIT_TRY(ensure(p, &p->wtab, wb + sizeof(double) * n_bands));
    double* cdev = (double*)((char*)p->wtab.p + wb);   // band centres after the table
    FIT_CUDA_CHECK(cudaMemcpyAsync(cdev, centers, sizeof(double) * n_bands, cudaMemcpyHostToDevice, p->stream));
    const unsigned dm = dims_mask ? dims_mask : ((1u << p->nd) - 1u);
    const unsigned nblk = (unsigned)((nw + 255) / 256);
    if (box)
      k_band_weights_box<<<nblk, 256, 0, p->stream>>>(p->g, p->kt, bK, bKX, bKY, dm, coord_f32, cdev, n_bands,
                                                      logwidth, (float*)p->wtab.p);
    else if (p->prec == 64)
      k_band_weights<double><<<nblk, 256, 0, p->stream>>>(p->g, p->kt, dm, coord_f32, cdev, n_bands, logwidth,
                                                          (double*)p->wtab.p);
    else
      k_band_weights<float><<<nblk, 256, 0, p->stream>>>(p->g, p->kt, dm, coord_f32, cdev, n_bands, logwidth,
                                                         (float*)p->wtab.p);
    FIT_LAUNCH_CHECK();
    p->wtab_key = key;
  }
  FIT_TRY(ensure(p, &p->outd, sizeof(double) * n_bands * n_bands));
  double* Td = (double*)p->outd.p;
  if (p->prec == 64) FIT_TRY(band_run<double>(p, ud, ad, n_bands, invariant, Td));
  else if (box) {   // FP32 cubic 3D plans of a fused size: every band through the live-box passes
    FIT_TRY(s2s_box_bands(p, ud, ad, n_bands, invariant, (const float*)p->wtab.p, Td));
    FIT_TRY(s2s_check(p));
  } else FIT_TRY(band_run<float>(p, ud, ad, n_bands, invariant, Td));
  std::vector<double> h((size_t)n_bands * n_bands);
  FIT_CUDA_CHECK(cudaMemcpyAsync(h.data(), Td, sizeof(double) * h.size(), cudaMemcpyDeviceToHost, p->stream));
  FIT_CUDA_CHECK(cudaStreamSynchronize(p->stream));
  double asym = 0.0;
  std::vector<double> nt(n_bands, 0.0);
  for (int n = 0; n < n_bands; ++n)
    for (int m = 0; m < n_bands; ++m) {
      nt[n] += h[(size_t)m * n_bands + n];
      const double a = fabs(h[(size_t)m * n_bands + n] + h[(size_t)n * n_bands + m]);
      if (a > asym) asym = a;
    }
  if (ptr_kind == FIT_PTR_DEVICE) {
    FIT_CUDA_CHECK(cudaMemcpyAsync(T_colmajor, h.data(), sizeof(double) * h.size(), cudaMemcpyHostToDevice,
                                   p->stream));
    if (net)
      FIT_CUDA_CHECK(cudaMemcpyAsync(net, nt.data(), sizeof(double) * n_bands, cudaMemcpyHostToDevice, p->stream));
    if (max_asym) FIT_CUDA_CHECK(cudaMemcpyAsync(max_asym, &asym, sizeof(double), cudaMemcpyHostToDevice, p->stream));
    FIT_CUDA_CHECK(cudaStreamSynchronize(p->stream));
  } else {
    memcpy(T_colmajor, h.data(), sizeof(double) * h.size());
    if (net) memcpy(net, nt.data(), sizeof(double) * n_bands);
    if (max_asym) *max_asym = asym;
  }
  return FIT_OK;
}
