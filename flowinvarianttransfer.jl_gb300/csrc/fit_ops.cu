// Pointwise and reduction kernels of the generic (any nd, any dealiasing, FP32/FP64) path:
// Hermitian gathers onto the transform grid, the physical-space product, effective carriers,
// deterministic-size shell binning, scatters back to the user layout, shell tables, and the
// helical / Helmholtz splits.
//
// Index maps between the transform grid M (half spectrum g = (g0 in [0, M0/2], g1, g2)) and the
// data grid N (full spectrum k):
//   * unpadded (M == N): k = g and its mirror k' = (-g) mod N;
//   * 3/2-padded: the data grid is embedded fftshift-centred, i.e. N-grid frequencies
//     f_d in [-floor(N_d/2), ceil(N_d/2)-1] (index N_d/2 -> -N_d/2) sit at the same signed
//     frequency of the M grid (ext/FlowInvariantTransferFFTWExt.jl:134-149).
// real(ifft(X)) equals the real transform of Herm(X)(g) = (X(g) + conj(X(-g)))/2, so every
// inverse-transform input is built as that Hermitian part of exactly the spectrum the
// reference forms (mask, band, derivative with its +N/2 Nyquist multiplier, embedding).
#include <math.h>
#include <stdio.h>

#include "fit_maps.cuh"
#include "fit_ops.cuh"

namespace fit {

static inline unsigned nblk(long n, int b) { return (unsigned)((n + b - 1) / b); }

// ---- Hermitian gather ------------------------------------------------------------------------

// One thread per half-spectrum mode, looping over the fields: the index maps, 2/3 predicate, shell
// lookups, wavenumbers and filter response are computed once per mode and reused by every field.
// CT is the arithmetic type: FP32 when both the source and the output are single precision (the
// result is rounded to FP32 anyway), FP64 otherwise.
template <typename V, typename CT>
__global__ void __launch_bounds__(256) k_gather(GridDesc g, KTab kt, GatherArgs a, V* out) {
  typedef typename Vec2<CT>::t C2;
  const long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (i >= g.Mhalf) return;
  int g0, g1, g2;
  decode_half(g, i, &g0, &g1, &g2);
  KIdx kk[2];
  map_pair(g, g0, g1, g2, &kk[0], &kk[1]);
  bool ok[2];
  CT kd[2][3], G[2] = {(CT)1, (CT)1};
  int sh[2] = {0, 0};
  bool any_band = false, any_filt = false;
#pragma unroll
  for (int f = 0; f < 16; ++f) {
    if (f < a.nfields) {
      any_band |= a.f[f].band > 0;
      any_filt |= a.f[f].filt != 0;
    }
  }
#pragma unroll
  for (int s = 0; s < 2; ++s) {
    ok[s] = kk[s].lin >= 0 && (!a.two_thirds || keep23(g, kk[s].k));
#pragma unroll
    for (int d = 0; d < 3; ++d) kd[s][d] = (d < g.nd && ok[s]) ? ktab_at<CT>(kt, d, kk[s].k[d]) : (CT)0;
    if (ok[s] && any_band) sh[s] = a.shell_full[kk[s].lin];
    if (ok[s] && any_filt) {   // |k| in FP64 for the filter response
      double k2 = 0.0;
      for (int d = 0; d < g.nd; ++d) {
        const double kv = kt.k[d][kk[s].k[d]];
        k2 += kv * kv;
      }
      G[s] = (CT)filter_response(a.filter_kind, sqrt(k2), a.ell);
    }
  }
  const CT sc = (CT)(0.5 * a.scale);
#pragma unroll
  for (int f = 0; f < 16; ++f) {   // unrolled: compile-time indices into the parameter block
    if (f >= a.nfields) break;
    const GatherField fd = a.f[f];
    CT ax = 0, ay = 0;
#pragma unroll
    for (int s = 0; s < 2; ++s) {
      if (!ok[s] || (fd.band > 0 && sh[s] != fd.band)) continue;
      const void* src = fd.src ? a.src[1] : a.src[0];
      const long idx = kk[s].lin + (fd.src ? a.src_comp_stride[1] : a.src_comp_stride[0]) * fd.comp;
      CT vx, vy;
      if (a.in_f64) {
        const double2 v = reinterpret_cast<const double2*>(src)[idx];
        vx = (CT)v.x;
        vy = (CT)v.y;
      } else {
        const float2 v = reinterpret_cast<const float2*>(src)[idx];
        vx = (CT)v.x;
        vy = (CT)v.y;
      }
      if (fd.deriv >= 0) {   // i k v
        const CT k = fd.deriv == 0 ? kd[s][0] : (fd.deriv == 1 ? kd[s][1] : kd[s][2]);
        const CT tx = -vy * k;
        vy = vx * k;
        vx = tx;
      }
      if (fd.filt) {
        vx *= G[s];
        vy *= G[s];
      }
      if (fd.wband > 0) {   // both conjugate modes share |k|, hence the weight of half mode i
        const long wi = (long)(fd.wband - 1) * g.Mhalf + i;
        const CT w = a.w_f64 ? (CT) reinterpret_cast<const double*>(a.wtab)[wi]
                             : (CT) reinterpret_cast<const float*>(a.wtab)[wi];
        vx *= w;
        vy *= w;
      }
      ax += vx;
      ay += s == 1 ? -vy : vy;
    }
    C2 r;
    r.x = ax * sc;
    r.y = ay * sc;
    V o;
    o.x = (typename Scal<V>::t)r.x;
    o.y = (typename Scal<V>::t)r.y;
    out[(long)f * g.Mhalf + i] = o;
  }
}

template <typename T>
int gather_half(const GridDesc& g, const KTab& kt, const GatherArgs& a, typename Vec2<T>::t* out, cudaStream_t st) {
  if (a.nfields <= 0 || a.nfields > 16) {
    fit_set_error("gather: bad field count %d", a.nfields);
    return FIT_ERR_ARG;
  }
  fit_prof_begin(PK_GATHER, (double)a.nfields * g.Mhalf * (sizeof(typename Vec2<T>::t) + 2.0 * (a.in_f64 ? 16 : 8)), st);
  if (sizeof(T) == 4 && !a.in_f64)
    k_gather<typename Vec2<T>::t, float><<<nblk(g.Mhalf, 256), 256, 0, st>>>(g, kt, a, out);
  else
    k_gather<typename Vec2<T>::t, double><<<nblk(g.Mhalf, 256), 256, 0, st>>>(g, kt, a, out);
  fit_prof_end(st);
  FIT_LAUNCH_CHECK();
  return FIT_OK;
}

// ---- physical-space product --------------------------------------------------------------------

template <typename T>
__global__ void k_product(const T* __restrict__ u, const T* __restrict__ grad, T* __restrict__ out, int nd, int M,
                          long n) {
  const long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (i >= n) return;
  T uu[3];
#pragma unroll
  for (int j = 0; j < 3; ++j) uu[j] = j < nd ? u[(long)j * n + i] : (T)0;
  for (int c = 0; c < M; ++c) {
    T s = (T)0;
#pragma unroll
    for (int j = 0; j < 3; ++j)
      if (j < nd) s += uu[j] * grad[(long)(c * nd + j) * n + i];
    out[(long)c * n + i] = s;
  }
}

template <typename T>
int product(const T* u, const T* grad, T* out, int nd, int M, long n, cudaStream_t st) {
  fit_prof_begin(PK_PRODUCT, (double)(nd + M * nd + M) * n * sizeof(T), st);
  k_product<T><<<nblk(n, 256), 256, 0, st>>>(u, grad, out, nd, M, n);
  fit_prof_end(st);
  FIT_LAUNCH_CHECK();
  return FIT_OK;
}

// For half-spectrum mode g: Ceff(g) = [A] C(kA) + [B] conj(C(kB)) such that the full N-grid shell
// sum sum_k Re(conj(C(k)) N(k)) equals sum_g Re(conj(Ceff(g)) Nhalf(g)) (N real in physical
// space, so N(-g) = conj(N(g))). Term A covers N-grid modes with non-negative x frequency, term
// B those with negative x frequency (never counted twice). seff = shell of those modes (equal for
// A and B: shells are symmetric under k -> -k), 0 when masked or absent.
template <typename V, typename CT>
__global__ void __launch_bounds__(256) k_ceff(GridDesc g, KTab kt, const void* car, int f64, long cs, int ncar, int inv,
                                              int two_thirds, const uint16_t* __restrict__ shell, V* ceff, int nce,
                                              uint16_t* seff) {
  typedef typename Vec2<CT>::t C2;
  const long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (i >= g.Mhalf) return;
  int g0, g1, g2;
  decode_half(g, i, &g0, &g1, &g2);
  KIdx kA, kB;
  map_pair(g, g0, g1, g2, &kA, &kB);
  bool A = kA.lin >= 0;
  bool B = kB.lin >= 0 && g0 >= 1 && (g.padded ? true : (2 * g0 < g.N[0]));
  uint16_t s = 0;
  if (A) s = shell[kA.lin];
  else if (B) s = shell[kB.lin];
  if (two_thirds) {
    const int* kk = A ? kA.k : kB.k;
    if ((A || B) && !keep23(g, kk)) s = 0;
  }
  C2 CA[3], CB[3];
#pragma unroll
  for (int c = 0; c < 3; ++c) CA[c] = CB[c] = mkc<C2>(0, 0);
  if (s != 0) {
    if (A) carrier_at_t<CT>(g, kt, car, f64, cs, ncar, inv, kA.lin, kA.k, CA);
    if (B) carrier_at_t<CT>(g, kt, car, f64, cs, ncar, inv, kB.lin, kB.k, CB);
  }
#pragma unroll
  for (int c = 0; c < 3; ++c)
    if (c < nce) {
      V o;
      o.x = (typename Scal<V>::t)(CA[c].x + CB[c].x);
      o.y = (typename Scal<V>::t)(CA[c].y - CB[c].y);
      ceff[(long)c * g.Mhalf + i] = o;
    }
  seff[i] = s;
}

template <typename T>
int effective_carrier(const GridDesc& g, const KTab& kt, const void* carrier, int in_f64, long comp_stride,
                      int ncomp_carrier, int invariant, int two_thirds, const uint16_t* shell_full,
                      typename Vec2<T>::t* ceff, int nceff, uint16_t* seff, cudaStream_t st) {
  if (nceff > 3 || ncomp_carrier > 3) {
    fit_set_error("effective carrier supports at most 3 components");
    return FIT_ERR_ARG;
  }
  fit_prof_begin(PK_CARRIER, (double)g.Mhalf * nceff * (sizeof(typename Vec2<T>::t) + 2.0 * (in_f64 ? 16 : 8)), st);
  if (sizeof(T) == 4 && !in_f64)
    k_ceff<typename Vec2<T>::t, float><<<nblk(g.Mhalf, 256), 256, 0, st>>>(
        g, kt, carrier, in_f64, comp_stride, ncomp_carrier, invariant, two_thirds, shell_full, ceff, nceff, seff);
  else
    k_ceff<typename Vec2<T>::t, double><<<nblk(g.Mhalf, 256), 256, 0, st>>>(
        g, kt, carrier, in_f64, comp_stride, ncomp_carrier, invariant, two_thirds, shell_full, ceff, nceff, seff);
  fit_prof_end(st);
  FIT_LAUNCH_CHECK();
  return FIT_OK;
}

// ---- shell binning ----------------------------------------------------------------------------
// Block-local FP64 bins in shared memory, per-block partials, then a fixed-order reduction over
// blocks. Runs of equal shells in consecutive lanes (modes along a row are ordered by |k|) are first
// summed by a log-step segmented warp reduction, so only each run's first lane touches the bins.
// The per-mode products and the in-warp run sums use CT: FP64 for FP64 data; FP32 for FP32 data
// (inputs carry FP32 rounding already; at most 32 terms per run), with every run sum accumulated
// in FP64 from there on. nset carrier sets (ceff_set_stride elements apart) are binned against the
// same N̂ in one pass.

template <typename V, typename CT>
__global__ void __launch_bounds__(256) k_bin(const V* __restrict__ nh, long bstride, int nb, const V* __restrict__ ceff,
                                             long cstride, int nset, int nc, const uint16_t* __restrict__ seff,
                                             long Mhalf, int nsh, double* __restrict__ partial) {
  extern __shared__ double bins[];
  const int nbins = nset * nb * nsh;
  for (int t = threadIdx.x; t < nbins; t += blockDim.x) bins[t] = 0.0;
  __syncthreads();
  const long step = (long)gridDim.x * blockDim.x;
  const long iters = (Mhalf + step - 1) / step;
  const unsigned lane = threadIdx.x & 31;
  for (long it = 0; it < iters; ++it) {
    const long i = it * step + blockIdx.x * (long)blockDim.x + threadIdx.x;
    const int s = (i < Mhalf) ? (int)seff[i] : 0;
    const int sr = __shfl_down_sync(0xffffffffu, s, 1);
    const int sl = __shfl_up_sync(0xffffffffu, s, 1);
    const unsigned same_right = __ballot_sync(0xffffffffu, lane < 31 && sr == s);
    const int run_end = __ffs(~same_right & (0xffffffffu << lane)) - 1;
    const bool head = lane == 0 || sl != s;
    for (int b = 0; b < nb; ++b) {
      V x[3];
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        x[c].x = x[c].y = 0;
        if (s && c < nc) x[c] = nh[b * bstride + (long)c * Mhalf + i];
      }
      for (int m = 0; m < nset; ++m) {
        CT v = 0;
        if (s) {
#pragma unroll
          for (int c = 0; c < 3; ++c) {
            if (c < nc) {
              const V cf = ceff[m * cstride + (long)c * Mhalf + i];
              v += (CT)cf.x * (CT)x[c].x + (CT)cf.y * (CT)x[c].y;
            }
          }
        }
#pragma unroll
        for (int off = 1; off < 32; off <<= 1) {
          const CT t = __shfl_down_sync(0xffffffffu, v, off);
          if ((int)lane + off <= run_end) v += t;
        }
        if (s && head) atomicAdd(&bins[(m * nb + b) * nsh + (s - 1)], (double)v);
      }
    }
  }
  __syncthreads();
  for (int t = threadIdx.x; t < nbins; t += blockDim.x) partial[(long)blockIdx.x * nbins + t] = bins[t];
}

// out[set][b*nsh + n] = sum over blocks of partial[block][(set*nb + b)*nsh + n]
__global__ void k_reduce_partials(const double* __restrict__ partial, int nblocks, int nbins, int per_set,
                                  BinOut out) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= nbins) return;
  double s = 0.0;
  for (int b = 0; b < nblocks; ++b) s += partial[(long)b * nbins + j];
  out.p[j / per_set][j % per_set] = s;
}

template <typename T>
int bin_density_multi(const GridDesc& g, const typename Vec2<T>::t* nh, long nh_batch_stride, int nb,
                      const typename Vec2<T>::t* ceff, long ceff_set_stride, int nset, int nc, const uint16_t* seff,
                      int nsh, double* partial, long partial_cap, const BinOut& out, cudaStream_t st,
                      long len) {
  typedef typename Vec2<T>::t V;
  const long L = len < 0 ? g.Mhalf : len;
  if (nset < 1 || nset > 8) {
    fit_set_error("binning: 1..8 carrier sets per pass (got %d)", nset);
    return FIT_ERR_ARG;
  }
  const int nbins = nset * nb * nsh;
  const size_t smem = sizeof(double) * nbins;
  if (smem > 96 * 1024) {
    fit_set_error("too many shell bins (%d) for one binning launch", nbins);
    return FIT_ERR_SIZE;
  }
  int nblocks = 2 * 152;
  const long needed = (L + 255) / 256;
  if (needed < nblocks) nblocks = (int)needed;
  if ((long)nblocks * nbins > partial_cap) nblocks = (int)(partial_cap / nbins);
  if (nblocks < 1) {
    fit_set_error("binning scratch too small");
    return FIT_ERR_SIZE;
  }
  const bool f32 = sizeof(T) == 4;
  if (smem > 48 * 1024) {
    cudaError_t e = f32 ? cudaFuncSetAttribute(k_bin<V, float>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem)
                        : cudaFuncSetAttribute(k_bin<V, double>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) {
      fit_set_error("cudaFuncSetAttribute failed: %s", cudaGetErrorString(e));
      return FIT_ERR_CUDA;
    }
  }
  fit_prof_begin(PK_BIN, (double)L * ((nb + nset) * nc * sizeof(V) + 2.0), st);
  if (f32)
    k_bin<V, float><<<nblocks, 256, smem, st>>>(nh, nh_batch_stride, nb, ceff, ceff_set_stride, nset, nc, seff, L,
                                               nsh, partial);
  else
    k_bin<V, double><<<nblocks, 256, smem, st>>>(nh, nh_batch_stride, nb, ceff, ceff_set_stride, nset, nc, seff,
                                                L, nsh, partial);
  fit_prof_end(st);
  FIT_LAUNCH_CHECK();
  k_reduce_partials<<<nblk(nbins, 128), 128, 0, st>>>(partial, nblocks, nbins, nb * nsh, out);
  FIT_LAUNCH_CHECK();
  return FIT_OK;
}

template <typename T>
int bin_density(const GridDesc& g, const typename Vec2<T>::t* nh, long nh_batch_stride, int nb,
                const typename Vec2<T>::t* ceff, int nc, const uint16_t* seff, int nsh, double* partial,
                long partial_cap, double* out, cudaStream_t st) {
  BinOut o;
  o.p[0] = out;
  return bin_density_multi<T>(g, nh, nh_batch_stride, nb, ceff, 0, 1, nc, seff, nsh, partial, partial_cap, o, st);
}

// ---- scatter to the full N-grid user layout ---------------------------------------------------

template <typename V>
__global__ void k_scatter(GridDesc g, const V* __restrict__ half, int nf, int two_thirds, void* out, int out_f64) {
  const long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (i >= g.Ntot) return;
  int k[3];
  k[0] = (int)(i % g.N[0]);
  const long r = i / g.N[0];
  k[1] = (int)(r % g.N[1]);
  k[2] = (int)(r / g.N[1]);
  const bool keep = !two_thirds || keep23(g, k);
  long src;
  bool cj;
  if (!g.padded) {
    if (k[0] < g.Mh0) {
      src = k[0] + (long)g.Mh0 * (k[1] + (long)g.M[1] * k[2]);
      cj = false;
    } else {
      src = (g.N[0] - k[0]) + (long)g.Mh0 * ((g.N[1] - k[1]) % g.N[1] + (long)g.M[1] * ((g.N[2] - k[2]) % g.N[2]));
      cj = true;
    }
  } else {
    int f[3];
    for (int d = 0; d < 3; ++d) f[d] = (2 * k[d] < g.N[d]) ? k[d] : k[d] - g.N[d];
    if (g.nd < 3) f[2] = 0;
    if (g.nd < 2) f[1] = 0;
    cj = f[0] < 0;
    if (cj) { f[0] = -f[0]; f[1] = -f[1]; f[2] = -f[2]; }
    src = f[0] + (long)g.Mh0 * (fmod_pos(f[1], g.M[1]) + (long)g.M[1] * fmod_pos(f[2], g.M[2]));
  }
  for (int c = 0; c < nf; ++c) {
    double2 v = make_double2(0, 0);
    if (keep) {
      const V h = half[(long)c * g.Mhalf + src];
      v = make_double2((double)h.x, cj ? -(double)h.y : (double)h.y);
    }
    if (out_f64) reinterpret_cast<double2*>(out)[(long)c * g.Ntot + i] = v;
    else reinterpret_cast<float2*>(out)[(long)c * g.Ntot + i] = make_float2((float)v.x, (float)v.y);
  }
}

template <typename T>
int scatter_full(const GridDesc& g, const typename Vec2<T>::t* half, int nf, int two_thirds, void* out, int out_f64,
                 cudaStream_t st) {
  k_scatter<typename Vec2<T>::t><<<nblk(g.Ntot, 256), 256, 0, st>>>(g, half, nf, two_thirds, out, out_f64);
  FIT_LAUNCH_CHECK();
  return FIT_OK;
}

// ---- shell tables ------------------------------------------------------------------------------
// kappa = sqrt(sum_{d in dims} k_d^2) accumulated in increasing d, every operation IEEE-rounded
// with no contraction (src/ShellBinning.jl:19-36), then the first n with
// edges[n] <= kappa < edges[n+1] (src/ShellBinning.jl:126-140). Edges are non-decreasing, so that
// n is the last edge <= kappa, found by binary search.

__global__ void k_shell(GridDesc g, KTab kt, unsigned dims, const double* __restrict__ edges, int ne, int f32,
                        uint16_t* out) {
  const long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (i >= g.Ntot) return;
  int k[3];
  k[0] = (int)(i % g.N[0]);
  const long r = i / g.N[0];
  k[1] = (int)(r % g.N[1]);
  k[2] = (int)(r / g.N[1]);
  double kap;
  if (!f32) {
    double s = 0.0;
    for (int d = 0; d < g.nd; ++d)
      if (dims & (1u << d)) {
        const double kd = kt.k[d][k[d]];
        s = __dadd_rn(s, __dmul_rn(kd, kd));
      }
    kap = __dsqrt_rn(s);
  } else {
    float s = 0.0f;
    for (int d = 0; d < g.nd; ++d)
      if (dims & (1u << d)) {
        const float kd = (float)kt.k[d][k[d]];
        s = __fadd_rn(s, __fmul_rn(kd, kd));
      }
    kap = (double)__fsqrt_rn(s);
  }
  int sh = 0;
  if (ne >= 2 && edges[0] <= kap) {
    int lo = 0, hi = ne - 1;   // invariant: edges[lo] <= kap; answer in [lo, hi]
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (edges[mid] <= kap) lo = mid; else hi = mid - 1;
    }
    if (lo < ne - 1 && kap < edges[lo + 1]) sh = lo + 1;
  }
  out[i] = (uint16_t)sh;
}

int shell_table(const GridDesc& g, const KTab& kt, unsigned dims_mask, const double* edges, int nedges, int coord_f32,
                uint16_t* out, cudaStream_t st) {
  if (nedges > 65536) {
    fit_set_error("at most 65535 shells are supported");
    return FIT_ERR_SIZE;
  }
  k_shell<<<nblk(g.Ntot, 256), 256, 0, st>>>(g, kt, dims_mask, edges, nedges, coord_f32, out);
  FIT_LAUNCH_CHECK();
  return FIT_OK;
}

__global__ void k_sh_i64(const uint16_t* __restrict__ sh, int64_t* out, long n) {
  const long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (i < n) out[i] = (int64_t)sh[i];
}

int shell_table_i64(const GridDesc& g, const uint16_t* sh, int64_t* out, cudaStream_t st) {
  k_sh_i64<<<nblk(g.Ntot, 256), 256, 0, st>>>(sh, out, g.Ntot);
  FIT_LAUNCH_CHECK();
  return FIT_OK;
}

// Rows (component c, z, y) of the kept box whose |signed y frequency| lies in [ya, yb), numbered
// (c, iz, j): j runs over the range's non-negative y values first, then its negative ones.
struct KeptRows {
  int N0, N1, N2, K0, K1, K2;
  int ya, yb;
  int npos, nyc;   // non-negative y values of the range, and all of them
  long nrows;
};

// element offset of row r's x = 0 in the column-major field
FIT_D long kept_row_base(const KeptRows& k, long r) {
  const int j = (int)(r % k.nyc);
  const long q = r / k.nyc;
  const int nz = 2 * k.K2 + 1;
  const int iz = (int)(q % nz), c = (int)(q / nz);
  const int y = j < k.npos ? k.ya + j : k.N1 - (k.yb - 1) + (j - k.npos);
  const int z = iz <= k.K2 ? iz : k.N2 - nz + iz;
  return (((long)c * k.N2 + z) * k.N1 + y) * (long)k.N0;
}

// The rows' kept elements (x in [0, K0] and [N0 - K0, N0)), flat over rows x elements so that a
// warp reads consecutive elements of a row; every thread has four loads in flight before its
// stores, so a small grid still keeps enough reads outstanding on the host link.
template <typename E>
__global__ void __launch_bounds__(256) k_copy_kept_rows(const E* __restrict__ src, E* __restrict__ dst, KeptRows k) {
  const int nx = 2 * k.K0 + 1;
  const long n = k.nrows * nx, stride = (long)gridDim.x * blockDim.x;
  for (long i0 = blockIdx.x * (long)blockDim.x + threadIdx.x; i0 < n; i0 += 4 * stride) {
    E v[4];
    long at[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const long i = i0 + u * stride;
      at[u] = -1;
      if (i < n) {
        const long r = i / nx;
        const int ix = (int)(i - r * nx);
        at[u] = kept_row_base(k, r) + (ix <= k.K0 ? ix : k.N0 - nx + ix);
        v[u] = src[at[u]];
      }
    }
#pragma unroll
    for (int u = 0; u < 4; ++u)
      if (at[u] >= 0) dst[at[u]] = v[u];
  }
}

// The same copy of 8-byte elements (complex64) in 16-byte pairs, for an even row length and 16-byte
// aligned arrays (every row starts on a 16-byte boundary): run A, x in [0, K0], in pairs from x = 0;
// run B, x in [N0 - K0, N0), in pairs ending at N0; the single elements left at odd run ends (x = K0
// when K0 + 1 is odd, x = N0 - K0 when that is odd) in a second loop.
__global__ void __launch_bounds__(256) k_copy_kept_rows_c64(const uint2* __restrict__ src, uint2* __restrict__ dst,
                                                            KeptRows k) {
  const int pA = (k.K0 + 1) >> 1, sB = k.N0 - k.K0, hB = sB & 1;
  const int pB = (k.N0 - sB - hB) >> 1, np = pA + pB, qB = (sB + hB) >> 1;   // qB: run B's first pair
  const long n = k.nrows * np, stride = (long)gridDim.x * blockDim.x;
  const long t0 = blockIdx.x * (long)blockDim.x + threadIdx.x;
  const uint4* s4 = reinterpret_cast<const uint4*>(src);
  uint4* d4 = reinterpret_cast<uint4*>(dst);
  for (long i0 = t0; i0 < n; i0 += 4 * stride) {
    uint4 v[4];
    long at[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const long i = i0 + u * stride;
      at[u] = -1;
      if (i < n) {
        const long r = i / np;
        const int t = (int)(i - r * np);
        at[u] = (kept_row_base(k, r) >> 1) + (t < pA ? t : qB + (t - pA));
        v[u] = s4[at[u]];
      }
    }
#pragma unroll
    for (int u = 0; u < 4; ++u)
      if (at[u] >= 0) d4[at[u]] = v[u];
  }
  const int s0 = (k.K0 + 1) & 1, ns = s0 + hB;
  for (long i = t0; i < k.nrows * ns; i += stride) {
    const long r = i / ns;
    const int w = (int)(i - r * ns);
    const long e = kept_row_base(k, r) + ((s0 && w == 0) ? k.K0 : sB);
    dst[e] = src[e];
  }
}

int copy_kept_rows(const void* src, void* dst, const int* N, int ncomp, int eb, int ya, int yb, int max_blocks,
                   cudaStream_t st) {
  KeptRows k;
  k.N0 = N[0];
  k.N1 = N[1];
  k.N2 = N[2];
  k.K0 = N[0] / 3 - 1;
  k.K1 = N[1] / 3 - 1;
  k.K2 = N[2] / 3 - 1;
  if (yb > k.K1 + 1) yb = k.K1 + 1;
  if (ya < 0) ya = 0;
  k.ya = ya;
  k.yb = yb;
  k.npos = yb - ya;
  k.nyc = k.npos + (yb - (ya > 1 ? ya : 1));
  k.nrows = (long)ncomp * (2 * k.K2 + 1) * k.nyc;
  if (k.K0 < 0 || k.npos <= 0 || k.nrows <= 0) return FIT_OK;
  const bool pairs = eb == 8 && N[0] % 2 == 0 && (((uintptr_t)src | (uintptr_t)dst) & 15) == 0;
  const long items = k.nrows * (pairs ? (long)k.K0 + 1 : 2L * k.K0 + 1);   // pairs: about (2 K0 + 1) / 2 a row
  long blocks = (items + 4 * 256 - 1) / (4 * 256);
  if (blocks > 152L * 64) blocks = 152L * 64;
  if (max_blocks > 0 && blocks > max_blocks) blocks = max_blocks;
  const unsigned nb = (unsigned)blocks;
  if (pairs)
    k_copy_kept_rows_c64<<<nb, 256, 0, st>>>((const uint2*)src, (uint2*)dst, k);
  else if (eb == 16)
    k_copy_kept_rows<uint4><<<nb, 256, 0, st>>>((const uint4*)src, (uint4*)dst, k);
  else
    k_copy_kept_rows<uint2><<<nb, 256, 0, st>>>((const uint2*)src, (uint2*)dst, k);
  FIT_LAUNCH_CHECK();
  return FIT_OK;
}

int copy_kept_box(const void* src, void* dst, const int* N, int ncomp, int eb, cudaStream_t st) {
  return copy_kept_rows(src, dst, N, ncomp, eb, 0, N[1] / 3, 0, st);
}

__global__ void k_sh_from_i64(const int64_t* __restrict__ idx, long n, int nsh, uint16_t* __restrict__ out,
                              unsigned long long* bad, unsigned* changed) {
  const long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int64_t v = idx[i];
  const bool ok = v >= 0 && v <= nsh;
  const uint16_t t = ok ? (uint16_t)v : (uint16_t)0;
  if (out[i] != t) {
    out[i] = t;
    *changed = 1u;
  }
  if (!ok) atomicMin(bad, (unsigned long long)i);
}

int shell_table_from_i64(const GridDesc& g, const int64_t* idx, int nsh, uint16_t* out, unsigned long long* bad,
                         unsigned* changed, cudaStream_t st) {
  k_sh_from_i64<<<nblk(g.Ntot, 256), 256, 0, st>>>(idx, g.Ntot, nsh, out, bad, changed);
  FIT_LAUNCH_CHECK();
  return FIT_OK;
}

// ---- per-mode density on the full grid ---------------------------------------------------------

__global__ void k_density_full(GridDesc g, KTab kt, const void* car, const void* nhat, int f64, int nc, int inv,
                               double* out) {
  const long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (i >= g.Ntot) return;
  int k[3];
  k[0] = (int)(i % g.N[0]);
  const long r = i / g.N[0];
  k[1] = (int)(r % g.N[1]);
  k[2] = (int)(r / g.N[1]);
  double2 C[3];
  carrier_at(g, kt, car, f64, g.Ntot, nc, inv, i, k, C);
  double t = 0.0;
  for (int c = 0; c < nc; ++c) {
    const double2 n = ld_c(nhat, f64, i + g.Ntot * c);
    t += C[c].x * n.x + C[c].y * n.y;
  }
  out[i] = t;
}

int density_full(const GridDesc& g, const KTab& kt, const void* carrier, const void* nhat, int in_f64, int ncomp,
                 int invariant, double* out, cudaStream_t st) {
  k_density_full<<<nblk(g.Ntot, 256), 256, 0, st>>>(g, kt, carrier, nhat, in_f64, ncomp, invariant, out);
  FIT_LAUNCH_CHECK();
  return FIT_OK;
}

// ---- decompositions ----------------------------------------------------------------------------

FIT_D void st_c(void* p, int f64, long i, double2 v) {
  if (f64) reinterpret_cast<double2*>(p)[i] = v;
  else reinterpret_cast<float2*>(p)[i] = make_float2((float)v.x, (float)v.y);
}

// Craya-Herring basis per mode, as src/Decomposition.jl:63-98 (reference vector z unless
// |khat_z| >= 0.9, then x; the mean mode carries nothing).
// Arithmetic in CT: FP32 for single-precision fields, FP64 otherwise. The split is invariant under
// the choice of the transverse pair (e1, e2): a rotation of the pair multiplies h+- by a phase and
// the coefficients by its conjugate.
// kept_only: modes outside the 2/3-kept box are neither read nor written (for consumers that
// never read them).
template <typename CT>
__global__ void __launch_bounds__(256) k_helical(GridDesc g, KTab kt, const void* u, int f64, void* up, void* um,
                                                 int kept_only) {
  typedef typename Vec2<CT>::t C2;
  const long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (i >= g.Ntot) return;
  int k[3];
  decode_full(g, i, k);
  if (kept_only && !keep23(g, k)) return;
  const CT kx = ktab_at<CT>(kt, 0, k[0]), ky = ktab_at<CT>(kt, 1, k[1]), kz = ktab_at<CT>(kt, 2, k[2]);
  const CT kk = sqrt(kx * kx + ky * ky + kz * kz);
  const long n = g.Ntot;
  C2 P[3], Mv[3];
  if (kk == (CT)0) {
#pragma unroll
    for (int c = 0; c < 3; ++c) P[c] = Mv[c] = mkc<C2>(0, 0);
  } else {
    const CT hx = kx / kk, hy = ky / kk, hz = kz / kk;
    CT rx = 0, ry = 0, rz = 1;
    if (!(fabs(hz) < (CT)0.9)) { rx = 1; rz = 0; }
    CT e1x = hy * rz - hz * ry, e1y = hz * rx - hx * rz, e1z = hx * ry - hy * rx;
    const CT n1 = sqrt(e1x * e1x + e1y * e1y + e1z * e1z);
    e1x /= n1; e1y /= n1; e1z /= n1;
    const CT e2x = hy * e1z - hz * e1y, e2y = hz * e1x - hx * e1z, e2z = hx * e1y - hy * e1x;
    const C2 u1 = ld_ct<CT>(u, f64, i), u2 = ld_ct<CT>(u, f64, i + n), u3 = ld_ct<CT>(u, f64, i + 2 * n);
    const C2 ue1 = mkc<C2>(u1.x * e1x + u2.x * e1y + u3.x * e1z, u1.y * e1x + u2.y * e1y + u3.y * e1z);
    const C2 ue2 = mkc<C2>(u1.x * e2x + u2.x * e2y + u3.x * e2z, u1.y * e2x + u2.y * e2y + u3.y * e2z);
    const CT is2 = (CT)0.70710678118654752440;
    // u+ coefficient (ue1 - i ue2)/sqrt2, u- coefficient (ue1 + i ue2)/sqrt2
    const C2 upc = mkc<C2>((ue1.x + ue2.y) * is2, (ue1.y - ue2.x) * is2);
    const C2 umc = mkc<C2>((ue1.x - ue2.y) * is2, (ue1.y + ue2.x) * is2);
    const CT e1[3] = {e1x, e1y, e1z}, e2[3] = {e2x, e2y, e2z};
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const C2 hp = mkc<C2>(e1[c] * is2, e2[c] * is2);    // (e1 + i e2)/sqrt2
      const C2 hm = mkc<C2>(e1[c] * is2, -e2[c] * is2);   // (e1 - i e2)/sqrt2
      P[c] = mkc<C2>(upc.x * hp.x - upc.y * hp.y, upc.x * hp.y + upc.y * hp.x);
      Mv[c] = mkc<C2>(umc.x * hm.x - umc.y * hm.y, umc.x * hm.y + umc.y * hm.x);
    }
  }
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    if (f64) {
      reinterpret_cast<double2*>(up)[i + n * c] = make_double2((double)P[c].x, (double)P[c].y);
      reinterpret_cast<double2*>(um)[i + n * c] = make_double2((double)Mv[c].x, (double)Mv[c].y);
    } else {
      reinterpret_cast<float2*>(up)[i + n * c] = make_float2((float)P[c].x, (float)P[c].y);
      reinterpret_cast<float2*>(um)[i + n * c] = make_float2((float)Mv[c].x, (float)Mv[c].y);
    }
  }
}

// Toroidal / poloidal split per mode, as src/Decomposition.jl:107-141: e1 = khat x zhat normalised
// (horizontal, toroidal direction), e2 = khat x e1 (poloidal); for k parallel to zhat the pair is
// (xhat, yhat); tor = (u . e1) e1, pol = (u . e2) e2; the mean mode carries nothing. Arithmetic in
// CT (the field's precision, as the reference computes in its element type).
template <typename CT>
__global__ void __launch_bounds__(256) k_toroidal(GridDesc g, KTab kt, const void* u, int f64, void* tor, void* pol,
                                                  int kept_only) {
  typedef typename Vec2<CT>::t C2;
  const long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (i >= g.Ntot) return;
  int k[3];
  decode_full(g, i, k);
  if (kept_only && !keep23(g, k)) return;
  const CT kx = (CT)kt.k[0][k[0]], ky = (CT)kt.k[1][k[1]], kz = (CT)kt.k[2][k[2]];
  const CT kk = sqrt(kx * kx + ky * ky + kz * kz);
  const long n = g.Ntot;
  C2 T[3], Pv[3];
#pragma unroll
  for (int c = 0; c < 3; ++c) T[c] = Pv[c] = mkc<C2>(0, 0);
  if (kk != (CT)0) {
    const CT hx = kx / kk, hy = ky / kk, hz = kz / kk;
    const CT kperp = sqrt(kx * kx + ky * ky);
    CT e1x = 1, e1y = 0, e1z = 0, e2x = 0, e2y = 1, e2z = 0;
    if (kperp > (CT)0) {
      e1x = hy;   // khat x zhat = (hy, -hx, 0)
      e1y = -hx;
      e1z = 0;
      const CT n1 = sqrt(e1x * e1x + e1y * e1y + e1z * e1z);
      e1x /= n1;
      e1y /= n1;
      e1z /= n1;
      e2x = hy * e1z - hz * e1y;
      e2y = hz * e1x - hx * e1z;
      e2z = hx * e1y - hy * e1x;
    }
    const C2 u1 = ld_ct<CT>(u, f64, i), u2 = ld_ct<CT>(u, f64, i + n), u3 = ld_ct<CT>(u, f64, i + 2 * n);
    const C2 c1 = mkc<C2>(u1.x * e1x + u2.x * e1y + u3.x * e1z, u1.y * e1x + u2.y * e1y + u3.y * e1z);
    const C2 c2 = mkc<C2>(u1.x * e2x + u2.x * e2y + u3.x * e2z, u1.y * e2x + u2.y * e2y + u3.y * e2z);
    const CT e1[3] = {e1x, e1y, e1z}, e2[3] = {e2x, e2y, e2z};
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      T[c] = mkc<C2>(c1.x * e1[c], c1.y * e1[c]);
      Pv[c] = mkc<C2>(c2.x * e2[c], c2.y * e2[c]);
    }
  }
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    if (f64) {
      reinterpret_cast<double2*>(tor)[i + n * c] = make_double2((double)T[c].x, (double)T[c].y);
      reinterpret_cast<double2*>(pol)[i + n * c] = make_double2((double)Pv[c].x, (double)Pv[c].y);
    } else {
      reinterpret_cast<float2*>(tor)[i + n * c] = make_float2((float)T[c].x, (float)T[c].y);
      reinterpret_cast<float2*>(pol)[i + n * c] = make_float2((float)Pv[c].x, (float)Pv[c].y);
    }
  }
}

int toroidal_split(const GridDesc& g, const KTab& kt, const void* u, int in_f64, void* tor, void* pol, cudaStream_t st,
                   bool kept_only) {
  if (g.nd != 3) {
    fit_set_error("ToroidalPoloidalDecomposition is defined in 3D only (got nd=%d).", g.nd);
    return FIT_ERR_ARG;
  }
  if (in_f64) k_toroidal<double><<<nblk(g.Ntot, 256), 256, 0, st>>>(g, kt, u, in_f64, tor, pol, kept_only ? 1 : 0);
  else k_toroidal<float><<<nblk(g.Ntot, 256), 256, 0, st>>>(g, kt, u, in_f64, tor, pol, kept_only ? 1 : 0);
  FIT_LAUNCH_CHECK();
  return FIT_OK;
}

int helical_split(const GridDesc& g, const KTab& kt, const void* u, int in_f64, void* up, void* um, cudaStream_t st,
                  bool kept_only) {
  if (g.nd != 3) {
    fit_set_error("HelicalDecomposition is defined in 3D only (got nd=%d).", g.nd);
    return FIT_ERR_ARG;
  }
  if (in_f64) k_helical<double><<<nblk(g.Ntot, 256), 256, 0, st>>>(g, kt, u, in_f64, up, um, kept_only ? 1 : 0);
  else k_helical<float><<<nblk(g.Ntot, 256), 256, 0, st>>>(g, kt, u, in_f64, up, um, kept_only ? 1 : 0);
  FIT_LAUNCH_CHECK();
  return FIT_OK;
}

__global__ void k_helmholtz(GridDesc g, KTab kt, const void* u, int f64, void* rot, void* dv) {
  const long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (i >= g.Ntot) return;
  const int k0 = (int)(i % g.N[0]), k1 = (int)(i / g.N[0]);
  const double kx = kt.k[0][k0], ky = kt.k[1][k1];
  const double k2 = kx * kx + ky * ky;
  const long n = g.Ntot;
  const double2 a = ld_c(u, f64, i), b = ld_c(u, f64, i + n);
  double2 dx = make_double2(0, 0), dy = make_double2(0, 0);
  if (k2 > 0) {
    const double2 kd = make_double2((kx * a.x + ky * b.x) / k2, (kx * a.y + ky * b.y) / k2);
    dx = make_double2(kx * kd.x, kx * kd.y);
    dy = make_double2(ky * kd.x, ky * kd.y);
  }
  st_c(dv, f64, i, dx);
  st_c(dv, f64, i + n, dy);
  st_c(rot, f64, i, make_double2(a.x - dx.x, a.y - dx.y));
  st_c(rot, f64, i + n, make_double2(b.x - dy.x, b.y - dy.y));
}

int helmholtz_split(const GridDesc& g, const KTab& kt, const void* u, int in_f64, void* rot, void* div,
                    cudaStream_t st) {
  if (g.nd != 2) {
    fit_set_error("Helmholtz decomposition currently supports 2D fields only.");
    return FIT_ERR_ARG;
  }
  k_helmholtz<<<nblk(g.Ntot, 256), 256, 0, st>>>(g, kt, u, in_f64, rot, div);
  FIT_LAUNCH_CHECK();
  return FIT_OK;
}

__global__ void k_convert(const void* in, int in_f64, void* out, int out_f64, long n) {
  const long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (i >= n) return;
  st_c(out, out_f64, i, ld_c(in, in_f64, i));
}

int convert_complex(const void* in, int in_f64, void* out, int out_f64, long n, cudaStream_t st) {
  k_convert<<<nblk(n, 256), 256, 0, st>>>(in, in_f64, out, out_f64, n);
  FIT_LAUNCH_CHECK();
  return FIT_OK;
}

// ---- explicit instantiations -------------------------------------------------------------------
template int gather_half<float>(const GridDesc&, const KTab&, const GatherArgs&, float2*, cudaStream_t);
template int gather_half<double>(const GridDesc&, const KTab&, const GatherArgs&, double2*, cudaStream_t);
template int product<float>(const float*, const float*, float*, int, int, long, cudaStream_t);
template int product<double>(const double*, const double*, double*, int, int, long, cudaStream_t);
template int effective_carrier<float>(const GridDesc&, const KTab&, const void*, int, long, int, int, int,
                                      const uint16_t*, float2*, int, uint16_t*, cudaStream_t);
template int effective_carrier<double>(const GridDesc&, const KTab&, const void*, int, long, int, int, int,
                                       const uint16_t*, double2*, int, uint16_t*, cudaStream_t);
template int bin_density_multi<float>(const GridDesc&, const float2*, long, int, const float2*, long, int, int,
                                      const uint16_t*, int, double*, long, const BinOut&, cudaStream_t, long);
template int bin_density_multi<double>(const GridDesc&, const double2*, long, int, const double2*, long, int, int,
                                       const uint16_t*, int, double*, long, const BinOut&, cudaStream_t, long);
template int bin_density<float>(const GridDesc&, const float2*, long, int, const float2*, int, const uint16_t*, int,
                                double*, long, double*, cudaStream_t);
template int bin_density<double>(const GridDesc&, const double2*, long, int, const double2*, int, const uint16_t*,
                                 int, double*, long, double*, cudaStream_t);
template int scatter_full<float>(const GridDesc&, const float2*, int, int, void*, int, cudaStream_t);
template int scatter_full<double>(const GridDesc&, const double2*, int, int, void*, int, cudaStream_t);

}  // namespace fit
