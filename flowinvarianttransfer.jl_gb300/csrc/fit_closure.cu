// Coarse-graining flux and the forced Navier-Stokes evolver (the data path of the learned closure).
//
// Coarse-graining flux (restated in n-D; the reference computes it in 2D through the un-vendored
// CoarseGrainingEnergyFluxes.jl, src/CoarseGrainingFlux.jl:60-72, ext/FlowInvariantTransferCGEFExt.jl):
//   u(x)      = sum_k û(k) e^{ikx}            (û = fft(u)/Np, so this is the physical field)
//   ū_i       = G_ell * u_i,                    G = filter_response(kind, |k|, ell) (src/Filters.jl:19-26)
//   A_ij      = d_j ū_i                         (filtered velocity-gradient tensor)
//   tau_ij    = G_ell * (u_i u_j) - ū_i ū_j      (subfilter stress)
//   Pi_ell(x) = -tau_ij S_ij,  S_ij = (A_ij + A_ji)/2
// Forced Navier-Stokes (SSP-RK3, Shu-Osher) on the spectral state û:
//   dû/dt = -P[N̂(û)] - nu |k|^2 û + alpha û [0 < |k| <= kf],  P = Leray projector,
//   alpha = power / (2 E_f),  E_f = 1/2 sum_{0<|k|<=kf} |û|^2  (constant power injection);
// N̂ = Np^2 * (this library's nonlinear term): with the coefficient convention û = fft(u)/Np the
// nonlinear term (src/NonlinearTerm.jl, ext/FlowInvariantTransferFFTWExt.jl:61-121) transforms
// ifft(û) = u/Np, so it returns the physical advection coefficients divided by Np^2. The state is
// kept on the retained (2/3) modes.
#include <math.h>
#include <string.h>

#include "fit_gb300.h"
#include "fit_maps.cuh"
#include "fit_plan.cuh"

namespace fit {

static inline unsigned cl_blk(long n, int b) { return (unsigned)((n + b - 1) / b); }

template <typename V>
__global__ void k_filter_half(GridDesc g, KTab kt, V* h, int nf, int kind, double ell) {
  const long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (i >= g.Mhalf) return;
  int g0, g1, g2;
  decode_half(g, i, &g0, &g1, &g2);
  const int kk[3] = {g0, g1, g2};
  double k2 = 0.0;
  for (int d = 0; d < g.nd; ++d) {
    const double kd = kt.k[d][kk[d]];
    k2 += kd * kd;
  }
  const double G = filter_response(kind, sqrt(k2), ell);
  for (int f = 0; f < nf; ++f) {
    V v = h[(long)f * g.Mhalf + i];
    v.x *= G;
    v.y *= G;
    h[(long)f * g.Mhalf + i] = v;
  }
}

// the six products u_i u_j (i <= j, order 00 11 22 01 02 12 in 3D; 00 11 01 in 2D)
template <typename T>
__global__ void k_cg_products(const T* __restrict__ u, T* __restrict__ p, int nd, long n) {
  const long x = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (x >= n) return;
  T v[3];
  for (int i = 0; i < nd; ++i) v[i] = u[(long)i * n + x];
  int q = 0;
  for (int i = 0; i < nd; ++i) p[(long)(q++) * n + x] = v[i] * v[i];
  for (int i = 0; i < nd; ++i)
    for (int j = i + 1; j < nd; ++j) p[(long)(q++) * n + x] = v[i] * v[j];
}

// tau = filtered products - ū ū, Pi = -tau : S; optional copies of A and tau (plan precision).
template <typename T>
__global__ void k_cg_flux(const T* __restrict__ ub, const T* __restrict__ A, const T* __restrict__ fp, int nd,
                          long n, T* Pi, T* A_out, T* tau_out, double* mean) {
  const long x = blockIdx.x * (long)blockDim.x + threadIdx.x;
  double pv = 0.0;
  if (x < n) {
    T b[3];
    for (int i = 0; i < nd; ++i) b[i] = ub[(long)i * n + x];
    int q = 0;
    double pi = 0.0;
    for (int i = 0; i < nd; ++i) {
      const double tau = (double)fp[(long)q * n + x] - (double)b[i] * (double)b[i];
      if (tau_out) tau_out[(long)q * n + x] = (T)tau;
      pi -= tau * (double)A[(long)(i * nd + i) * n + x];
      ++q;
    }
    for (int i = 0; i < nd; ++i)
      for (int j = i + 1; j < nd; ++j) {
        const double tau = (double)fp[(long)q * n + x] - (double)b[i] * (double)b[j];
        if (tau_out) tau_out[(long)q * n + x] = (T)tau;
        pi -= tau * ((double)A[(long)(i * nd + j) * n + x] + (double)A[(long)(j * nd + i) * n + x]);
        ++q;
      }
    if (A_out)
      for (int c = 0; c < nd * nd; ++c) A_out[(long)c * n + x] = A[(long)c * n + x];
    Pi[x] = (T)pi;
    pv = pi;
  }
  // block sum of Pi for the mean
  for (int o = 16; o > 0; o >>= 1) pv += __shfl_down_sync(0xffffffffu, pv, o);
  __shared__ double ws[32];
  if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = pv;
  __syncthreads();
  if (threadIdx.x < 32) {
    double s = threadIdx.x < (blockDim.x >> 5) ? ws[threadIdx.x] : 0.0;
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if (threadIdx.x == 0) atomicAdd(mean, s);
  }
}

template <typename T>
static int cg_run(fit_plan* p, const void* ud, double ell, int kind, void* Pi, void* A_out, void* tau_out,
                  double* mean_dev) {
  typedef typename Vec2<T>::t V;
  const GridDesc& g = p->g;
  const int nd = p->nd;
  const int np = nd * (nd + 1) / 2;
  const long n = g.Mtot;
  FIT_TRY(ensure(p, &p->hs, sizeof(V) * 9 * g.Mhalf));
  FIT_TRY(ensure(p, &p->ph, sizeof(T) * (2 * nd + nd * nd + np) * n));
  FIT_TRY(ensure(p, &p->nph, sizeof(T) * np * n));
  FIT_TRY(ensure(p, &p->nh, sizeof(V) * np * g.Mhalf));
  V* hs = (V*)p->hs.p;
  T* ph = (T*)p->ph.p;
  T* u = ph;
  T* ub = ph + (long)nd * n;
  T* A = ph + 2L * nd * n;
  T* fp = ph + (2L * nd + nd * nd) * n;
  GatherArgs a;
  memset(&a, 0, sizeof(a));
  a.src[0] = ud;
  a.src_comp_stride[0] = g.Ntot;
  a.in_f64 = p->io_f64;
  a.scale = 1.0;
  a.filter_kind = kind;
  a.ell = ell;
  a.nfields = nd;
  for (int i = 0; i < nd; ++i) a.f[i] = GatherField{0, i, -1, 0, 0};
  FIT_TRY(gather_half<T>(g, p->kt, a, hs, p->stream));
  FIT_TRY(inverse_nd<T>(hs, u, g, p->ax, nd, (T)1, p->stream));
  // Filter and differentiate the spectrum of the real field u (Hermitian by construction), so that
  // an input that is not Hermitian on the Nyquist planes (a Leray split with +N/2 there) gives the
  // flux of the real velocity it stands for.
  FIT_TRY(ensure(p, &p->out_c2, sizeof(V) * nd * g.Ntot));
  FIT_TRY(forward_nd<T>(u, (V*)p->nh.p, g, p->ax, nd, (T)(1.0 / (double)n), p->stream));
  FIT_TRY(scatter_full<T>(g, (const V*)p->nh.p, nd, 0, p->out_c2.p, sizeof(T) == 8, p->stream));
  a.src[0] = p->out_c2.p;
  a.in_f64 = sizeof(T) == 8;
  for (int i = 0; i < nd; ++i) a.f[i] = GatherField{0, i, -1, 0, 1};
  FIT_TRY(gather_half<T>(g, p->kt, a, hs, p->stream));
  FIT_TRY(inverse_nd<T>(hs, ub, g, p->ax, nd, (T)1, p->stream));
  a.nfields = nd * nd;
  for (int i = 0; i < nd; ++i)
    for (int j = 0; j < nd; ++j) a.f[i * nd + j] = GatherField{0, i, j, 0, 1};
  FIT_TRY(gather_half<T>(g, p->kt, a, hs, p->stream));
  FIT_TRY(inverse_nd<T>(hs, A, g, p->ax, nd * nd, (T)1, p->stream));
  k_cg_products<T><<<cl_blk(n, 256), 256, 0, p->stream>>>(u, (T*)p->nph.p, nd, n);
  FIT_LAUNCH_CHECK();
  FIT_TRY(forward_nd<T>((const T*)p->nph.p, (V*)p->nh.p, g, p->ax, np, (T)(1.0 / (double)n), p->stream));
  k_filter_half<V><<<cl_blk(g.Mhalf, 256), 256, 0, p->stream>>>(g, p->kt, (V*)p->nh.p, np, kind, ell);
  FIT_LAUNCH_CHECK();
  FIT_TRY(inverse_nd<T>((V*)p->nh.p, fp, g, p->ax, np, (T)1, p->stream));
  FIT_CUDA_CHECK(cudaMemsetAsync(mean_dev, 0, sizeof(double), p->stream));
  k_cg_flux<T><<<cl_blk(n, 256), 256, 0, p->stream>>>(ub, A, fp, nd, n, (T*)Pi, (T*)A_out, (T*)tau_out, mean_dev);
  FIT_LAUNCH_CHECK();
  return FIT_OK;
}

// real element-type conversion (user io type -> plan precision)
template <typename S, typename T>
__global__ void k_convert_real(const S* __restrict__ in, T* __restrict__ out, long n) {
  const long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (i < n) out[i] = (T)in[i];
}

// û = fft(u)/Np of nf real physical fields (x fastest), full N-grid spectrum in the io type.
template <typename T>
static int forward_spectrum(fit_plan* p, const void* u_dev, void* out_dev) {
  typedef typename Vec2<T>::t V;
  const GridDesc& g = p->g;
  const int nf = p->M;
  const long n = g.Mtot;
  FIT_TRY(ensure(p, &p->nh, sizeof(V) * nf * g.Mhalf));
  const bool same = (p->io_f64 != 0) == (sizeof(T) == 8);
  if (same) {   // the real fields are read in place; the z pass writes the full spectrum itself
    const int rc = forward_nd_full<T>((const T*)u_dev, (V*)p->nh.p, (V*)out_dev, g, p->ax, nf,
                                      (T)(1.0 / (double)n), p->stream);
    if (rc != 1) return rc;
  }
  FIT_TRY(ensure(p, &p->ph, sizeof(T) * nf * n));
  T* ph = (T*)p->ph.p;
  if (p->io_f64 && sizeof(T) == 4) {
    k_convert_real<double, T><<<cl_blk(nf * n, 256), 256, 0, p->stream>>>((const double*)u_dev, ph, nf * n);
    FIT_LAUNCH_CHECK();
  } else if (!p->io_f64 && sizeof(T) == 8) {
    k_convert_real<float, T><<<cl_blk(nf * n, 256), 256, 0, p->stream>>>((const float*)u_dev, ph, nf * n);
    FIT_LAUNCH_CHECK();
  } else {
    FIT_CUDA_CHECK(cudaMemcpyAsync(ph, u_dev, sizeof(T) * nf * n, cudaMemcpyDeviceToDevice, p->stream));
  }
  FIT_TRY(forward_nd<T>(ph, (V*)p->nh.p, g, p->ax, nf, (T)(1.0 / (double)n), p->stream));
  FIT_TRY(scatter_full<T>(g, (const V*)p->nh.p, nf, 0, out_dev, p->io_f64, p->stream));
  return FIT_OK;
}

// ---- forced Navier-Stokes ---------------------------------------------------------------------

// Energy of the forced band 0 < |k| <= kf, summed in FP64 over the modes of a box of signed
// indices lo_d .. lo_d + len_d - 1 per axis that holds every |k_d| <= kf (each index once): only that
// corner of the spectrum is read.
template <typename CT>
__global__ void k_ns_forced_energy(GridDesc g, KTab kt, const void* u, int f64, int nc, double kf, int3 lo, int3 len,
                                   double* ef) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  double e = 0.0;
  if (t < len.x * len.y * len.z) {
    int k[3] = {t % len.x + lo.x, (t / len.x) % len.y + lo.y, t / (len.x * len.y) + lo.z};
    {
#pragma unroll
      for (int d = 0; d < 3; ++d) k[d] = k[d] < 0 ? k[d] + g.N[d] : k[d];
      double k2 = 0.0;   // the band test in FP64, as the reference's
      for (int d = 0; d < g.nd; ++d) k2 += kt.k[d][k[d]] * kt.k[d][k[d]];
      const long i = k[0] + (long)g.N[0] * (k[1] + (long)g.N[1] * k[2]);
      if (k2 > 0.0 && k2 <= kf * kf)
        for (int c = 0; c < nc; ++c) {
          const double2 v = ld_c(u, f64, i + g.Ntot * c);
          e += 0.5 * (v.x * v.x + v.y * v.y);
        }
    }
  }
  for (int o = 16; o > 0; o >>= 1) e += __shfl_down_sync(0xffffffffu, e, o);
  __shared__ double ws[32];
  if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = e;
  __syncthreads();
  if (threadIdx.x < 32) {
    double sum = threadIdx.x < (blockDim.x >> 5) ? ws[threadIdx.x] : 0.0;
    for (int o = 16; o > 0; o >>= 1) sum += __shfl_down_sync(0xffffffffu, sum, o);
    if (threadIdx.x == 0) atomicAdd(ef, sum);
  }
}

// out = a*u0 + b*(uin + dt*L(uin)), L = -P[N] - nu k^2 uin + alpha uin [0<|k|<=kf]; the state is
// restricted to the retained (2/3) modes. CT: FP32 for single-precision fields (per-mode work, no
// sums), FP64 otherwise.
template <typename CT>
__global__ void k_ns_update(GridDesc g, KTab kt, const void* u0, const void* uin, const void* Nh, void* out, int f64,
                            int nc, double a, double b, double dt, double nu, double kf, double power,
                            const double* ef, int two_thirds, double nscale, int3 fm) {
  typedef typename Vec2<CT>::t C2;
  const long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (i >= g.Ntot) return;
  int kidx[3];
  decode_full(g, i, kidx);
  CT kv[3];
#pragma unroll
  for (int d = 0; d < 3; ++d) kv[d] = d < g.nd ? ktab_at<CT>(kt, d, kidx[d]) : (CT)0;
  const CT k2 = kv[0] * kv[0] + kv[1] * kv[1] + kv[2] * kv[2];
  const bool keep = !two_thirds || keep23(g, kidx);
  C2 nn[3], ui[3];
  CT kn_re = 0, kn_im = 0;
  const CT ns = (CT)nscale;
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    if (c >= nc) break;
    nn[c] = ld_ct<CT>(Nh, f64, i + g.Ntot * c);
    nn[c].x *= ns;
    nn[c].y *= ns;
    ui[c] = ld_ct<CT>(uin, f64, i + g.Ntot * c);
    kn_re += kv[c] * nn[c].x;
    kn_im += kv[c] * nn[c].y;
  }
  // forcing band 0 < |k| <= kf, tested in FP64 for the modes of its index box (|signed index| <= fm)
  bool forced = false;
  {
    const int fmv[3] = {fm.x, fm.y, fm.z};
    bool inbox = true;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      const int sd = 2 * kidx[d] < g.N[d] ? kidx[d] : kidx[d] - g.N[d];
      inbox = inbox && (sd <= fmv[d] && -sd <= fmv[d]);
    }
    if (inbox) {
      double kd2 = 0.0;
      for (int d = 0; d < g.nd; ++d) kd2 += kt.k[d][kidx[d]] * kt.k[d][kidx[d]];
      forced = kd2 > 0.0 && kd2 <= kf * kf;
    }
  }
  const CT alpha = (forced && *ef > 0.0) ? (CT)(power / (2.0 * *ef)) : (CT)0;
  const CT cb = (CT)b, cdt = (CT)dt, ca = (CT)a;
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    if (c >= nc) break;
    C2 pn = nn[c];
    if (k2 > (CT)0) {
      pn.x -= kv[c] * kn_re / k2;
      pn.y -= kv[c] * kn_im / k2;
    }
    const CT fac = -(CT)nu * k2 + alpha;
    C2 r;
    r.x = cb * (ui[c].x + cdt * (-pn.x + fac * ui[c].x));
    r.y = cb * (ui[c].y + cdt * (-pn.y + fac * ui[c].y));
    if (a != 0.0) {
      const C2 z = ld_ct<CT>(u0, f64, i + g.Ntot * c);
      r.x += ca * z.x;
      r.y += ca * z.y;
    }
    if (!keep || k2 == (CT)0) r.x = r.y = (CT)0;
    if (f64) reinterpret_cast<double2*>(out)[i + g.Ntot * c] = make_double2((double)r.x, (double)r.y);
    else reinterpret_cast<float2*>(out)[i + g.Ntot * c] = make_float2((float)r.x, (float)r.y);
  }
}

template <typename T>
static int ns_stage(fit_plan* p, const void* u0, const void* uin, void* out, void* Nfull, double a, double b,
                    double dt, double nu, double kf, double power, double* ef) {
  if (sizeof(T) == 4 && fz_box_ok(p)) {   // FP32 cubic 3D of a fused size: the live-box passes
    FIT_TRY(s2s_box_nonlinear_full(p, uin, Nfull));
  } else {
    FIT_TRY(nonlinear_half<T>(p, uin, uin, 0, false));
    FIT_TRY(scatter_full<T>(p->g, (const typename Vec2<T>::t*)p->nh.p, p->M, p->dealias == 1, Nfull, p->io_f64,
                            p->stream));
  }
  FIT_CUDA_CHECK(cudaMemsetAsync(ef, 0, sizeof(double), p->stream));
  int lo[3] = {0, 0, 0}, len[3] = {1, 1, 1};   // index box of the forced band, per axis
  for (int d = 0; d < p->nd; ++d) {
    const int N = p->g.N[d];
    int m = 0;
    while (m + 1 <= N / 2 && (fabs(p->ks_host[d][m + 1]) <= kf || fabs(p->ks_host[d][N - m - 1]) <= kf)) ++m;
    if (2 * m + 1 >= N) {   // the whole axis
      lo[d] = -(N / 2);
      len[d] = N;
    } else {
      lo[d] = -m;
      len[d] = 2 * m + 1;
    }
  }
  const int nbox = len[0] * len[1] * len[2];
  const bool f32 = sizeof(T) == 4;
  if (f32)
    k_ns_forced_energy<float><<<(nbox + 255) / 256, 256, 0, p->stream>>>(
        p->g, p->kt, uin, p->io_f64, p->M, kf, make_int3(lo[0], lo[1], lo[2]), make_int3(len[0], len[1], len[2]), ef);
  else
    k_ns_forced_energy<double><<<(nbox + 255) / 256, 256, 0, p->stream>>>(
        p->g, p->kt, uin, p->io_f64, p->M, kf, make_int3(lo[0], lo[1], lo[2]), make_int3(len[0], len[1], len[2]), ef);
  FIT_LAUNCH_CHECK();
  const double nsc = (double)p->g.Ntot * (double)p->g.Ntot;
  const int3 fm = make_int3(len[0] / 2, len[1] / 2, len[2] / 2);   // half-widths of the forced index box
  if (f32)
    k_ns_update<float><<<cl_blk(p->g.Ntot, 256), 256, 0, p->stream>>>(p->g, p->kt, u0, uin, Nfull, out, p->io_f64,
                                                                      p->M, a, b, dt, nu, kf, power, ef,
                                                                      p->dealias == 1, nsc, fm);
  else
    k_ns_update<double><<<cl_blk(p->g.Ntot, 256), 256, 0, p->stream>>>(p->g, p->kt, u0, uin, Nfull, out, p->io_f64,
                                                                       p->M, a, b, dt, nu, kf, power, ef,
                                                                       p->dealias == 1, nsc, fm);
  FIT_LAUNCH_CHECK();
  return FIT_OK;
}

}  // namespace fit

using namespace fit;

extern "C" int fit_coarse_graining_flux(fit_plan* p, const void* u_hat, double ell, int filter_kind, void* Pi,
                                        void* A_out, void* tau_out, double* Pi_mean, int ptr_kind) {
  if (!p || !u_hat || !Pi) {
    fit_set_error("NULL argument");
    return FIT_ERR_ARG;
  }
  if (p->M != p->nd || p->nd < 2 || p->g.padded) {
    fit_set_error("coarse-graining flux needs an nd-component velocity plan on an unpadded grid (nd >= 2)");
    return FIT_ERR_ARG;
  }
  if (!(ell > 0.0) || filter_kind < 0 || filter_kind > 2) {
    fit_set_error("filter scale must be positive and filter_kind in {0 sharp, 1 Gaussian, 2 top-hat}");
    return FIT_ERR_ARG;
  }
  const size_t cb = (p->io_f64 ? 16 : 8) * (size_t)p->g.Ntot * p->M;
  const void* ud = u_hat;
  if (ptr_kind != FIT_PTR_DEVICE) {
    FIT_TRY(ensure(p, &p->in_u, cb));
    FIT_CUDA_CHECK(cudaMemcpyAsync(p->in_u.p, u_hat, cb, cudaMemcpyHostToDevice, p->stream));
    ud = p->in_u.p;
  }
  const long n = p->g.Mtot;
  const size_t tb = p->prec == 64 ? 8 : 4;
  const int nd = p->nd, np = nd * (nd + 1) / 2;
  FIT_TRY(ensure(p, &p->outd, sizeof(double) * 2));
  double* mean_dev = (double*)p->outd.p;
  void *Pd = Pi, *Ad = A_out, *td = tau_out;
  if (ptr_kind != FIT_PTR_DEVICE) {
    FIT_TRY(ensure(p, &p->out_c, tb * n * (1 + (A_out ? nd * nd : 0) + (tau_out ? np : 0))));
    Pd = p->out_c.p;
    char* q = (char*)p->out_c.p + tb * n;
    if (A_out) {
      Ad = q;
      q += tb * nd * nd * n;
    }
    if (tau_out) td = q;
  }
  if (p->prec == 64) FIT_TRY(cg_run<double>(p, ud, ell, filter_kind, Pd, Ad, td, mean_dev));
  else FIT_TRY(cg_run<float>(p, ud, ell, filter_kind, Pd, Ad, td, mean_dev));
  if (ptr_kind != FIT_PTR_DEVICE) {
    FIT_CUDA_CHECK(cudaMemcpyAsync(Pi, Pd, tb * n, cudaMemcpyDeviceToHost, p->stream));
    if (A_out) FIT_CUDA_CHECK(cudaMemcpyAsync(A_out, Ad, tb * nd * nd * n, cudaMemcpyDeviceToHost, p->stream));
    if (tau_out) FIT_CUDA_CHECK(cudaMemcpyAsync(tau_out, td, tb * np * n, cudaMemcpyDeviceToHost, p->stream));
  }
  double s = 0.0;
  FIT_CUDA_CHECK(cudaMemcpyAsync(&s, mean_dev, sizeof(double), cudaMemcpyDeviceToHost, p->stream));
  FIT_CUDA_CHECK(cudaStreamSynchronize(p->stream));
  if (Pi_mean) *Pi_mean = s / (double)n;
  return FIT_OK;
}

extern "C" int fit_forward_spectrum(fit_plan* p, const void* u_phys, void* u_hat, int ptr_kind) {
  if (!p || !u_phys || !u_hat) {
    fit_set_error("NULL argument");
    return FIT_ERR_ARG;
  }
  if (p->g.padded) {
    fit_set_error("forward spectrum needs an unpadded plan");
    return FIT_ERR_ARG;
  }
  const size_t rb = (p->io_f64 ? 8 : 4) * (size_t)p->g.Ntot * p->M;
  const size_t cb = 2 * rb;
  const void* ud = u_phys;
  void* od = u_hat;
  if (ptr_kind != FIT_PTR_DEVICE) {
    FIT_TRY(ensure(p, &p->in_u, rb));
    FIT_TRY(ensure(p, &p->out_c, cb));
    FIT_CUDA_CHECK(cudaMemcpyAsync(p->in_u.p, u_phys, rb, cudaMemcpyHostToDevice, p->stream));
    ud = p->in_u.p;
    od = p->out_c.p;
  }
  if (p->prec == 64) FIT_TRY(forward_spectrum<double>(p, ud, od));
  else FIT_TRY(forward_spectrum<float>(p, ud, od));
  if (ptr_kind != FIT_PTR_DEVICE) FIT_CUDA_CHECK(cudaMemcpyAsync(u_hat, od, cb, cudaMemcpyDeviceToHost, p->stream));
  FIT_CUDA_CHECK(cudaStreamSynchronize(p->stream));
  return FIT_OK;
}

extern "C" int fit_ns_evolve(fit_plan* p, void* u_hat, int nsteps, double dt, double nu, double kf, double power,
                             int ptr_kind) {
  if (!p || !u_hat) {
    fit_set_error("NULL argument");
    return FIT_ERR_ARG;
  }
  if (p->M != p->nd || p->Dadv != p->nd || p->g.padded) {
    fit_set_error("the Navier-Stokes evolver needs an nd-component velocity plan (2/3 or no dealiasing)");
    return FIT_ERR_ARG;
  }
  if (nsteps < 0 || !(dt > 0.0) || nu < 0.0) {
    fit_set_error("need nsteps >= 0, dt > 0, nu >= 0");
    return FIT_ERR_ARG;
  }
  const size_t cb = (p->io_f64 ? 16 : 8) * (size_t)p->g.Ntot * p->M;
  void* u0 = u_hat;
  if (ptr_kind != FIT_PTR_DEVICE) {
    FIT_TRY(ensure(p, &p->in_u, cb));
    FIT_CUDA_CHECK(cudaMemcpyAsync(p->in_u.p, u_hat, cb, cudaMemcpyHostToDevice, p->stream));
    u0 = p->in_u.p;
  }
  FIT_TRY(ensure(p, &p->out_c, cb));
  FIT_TRY(ensure(p, &p->out_c2, cb));
  FIT_TRY(ensure(p, &p->outd, sizeof(double) * 2));
  void* u1 = p->out_c.p;
  void* Nf = p->out_c2.p;
  double* ef = (double*)p->outd.p;
  for (int s = 0; s < nsteps; ++s) {   // SSP-RK3 (Shu-Osher)
    if (p->prec == 64) {
      FIT_TRY(ns_stage<double>(p, u0, u0, u1, Nf, 0.0, 1.0, dt, nu, kf, power, ef));
      FIT_TRY(ns_stage<double>(p, u0, u1, u1, Nf, 0.75, 0.25, dt, nu, kf, power, ef));
      FIT_TRY(ns_stage<double>(p, u0, u1, u0, Nf, 1.0 / 3.0, 2.0 / 3.0, dt, nu, kf, power, ef));
    } else {
      FIT_TRY(ns_stage<float>(p, u0, u0, u1, Nf, 0.0, 1.0, dt, nu, kf, power, ef));
      FIT_TRY(ns_stage<float>(p, u0, u1, u1, Nf, 0.75, 0.25, dt, nu, kf, power, ef));
      FIT_TRY(ns_stage<float>(p, u0, u1, u0, Nf, 1.0 / 3.0, 2.0 / 3.0, dt, nu, kf, power, ef));
    }
  }
  if (ptr_kind != FIT_PTR_DEVICE) FIT_CUDA_CHECK(cudaMemcpyAsync(u_hat, u0, cb, cudaMemcpyDeviceToHost, p->stream));
  FIT_CUDA_CHECK(cudaStreamSynchronize(p->stream));
  return s2s_check(p);   // a bounded wait of the live-box x pass that gave up
}
