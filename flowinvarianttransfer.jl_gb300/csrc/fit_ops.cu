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

template <typename V>
__global__ void k_gather(GridDesc g, KTab kt, GatherArgs a, V* out) {
  const long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (i >= g.Mhalf) return;
  const GatherField f = a.f[blockIdx.y];
  int g0, g1, g2;
  decode_half(g, i, &g0, &g1, &g2);
  KIdx kk[2];
  map_pair(g, g0, g1, g2, &kk[0], &kk[1]);
  double2 acc = make_double2(0.0, 0.0);
#pragma unroll
  for (int s = 0; s < 2; ++s) {
    const KIdx& k = kk[s];
    if (k.lin < 0) continue;
    if (a.two_thirds && !keep23(g, k.k)) continue;
    if (f.band > 0 && a.shell_full[k.lin] != f.band) continue;
    double2 v = ld_c(a.src[f.src], a.in_f64, k.lin + a.src_comp_stride[f.src] * f.comp);
    if (f.deriv >= 0) v = dmul_i(v, kt.k[f.deriv][k.k[f.deriv]]);
    if (f.filt) {
      double k2 = 0.0;
      for (int d = 0; d < g.nd; ++d) {
        const double kd = kt.k[d][k.k[d]];
        k2 += kd * kd;
      }
      const double G = filter_response(a.filter_kind, sqrt(k2), a.ell);
      v.x *= G;
      v.y *= G;
    }
    if (s == 1) v.y = -v.y;
    acc.x += v.x;
    acc.y += v.y;
  }
  const double sc = 0.5 * a.scale;
  out[(long)blockIdx.y * g.Mhalf + i] = to_v<V>(make_double2(acc.x * sc, acc.y * sc));
}

template <typename T>
int gather_half(const GridDesc& g, const KTab& kt, const GatherArgs& a, typename Vec2<T>::t* out, cudaStream_t st) {
  if (a.nfields <= 0 || a.nfields > 16) {
    fit_set_error("gather: bad field count %d", a.nfields);
    return FIT_ERR_ARG;
  }
  dim3 grid(nblk(g.Mhalf, 256), a.nfields);
  fit_prof_begin(PK_GATHER, (double)a.nfields * g.Mhalf * (sizeof(typename Vec2<T>::t) + 2.0 * (a.in_f64 ? 16 : 8)), st);
  k_gather<typename Vec2<T>::t><<<grid, 256, 0, st>>>(g, kt, a, out);
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
  for (int j = 0; j < nd; ++j) uu[j] = u[(long)j * n + i];
  for (int c = 0; c < M; ++c) {
    T s = (T)0;
    for (int j = 0; j < nd; ++j) s += uu[j] * grad[(long)(c * nd + j) * n + i];
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
template <typename V>
__global__ void k_ceff(GridDesc g, KTab kt, const void* car, int f64, long cs, int ncar, int inv, int two_thirds,
                       const uint16_t* __restrict__ shell, V* ceff, int nce, uint16_t* seff) {
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
  double2 CA[3] = {make_double2(0, 0), make_double2(0, 0), make_double2(0, 0)};
  double2 CB[3] = {make_double2(0, 0), make_double2(0, 0), make_double2(0, 0)};
  if (s != 0) {
    if (A) carrier_at(g, kt, car, f64, cs, ncar, inv, kA.lin, kA.k, CA);
    if (B) carrier_at(g, kt, car, f64, cs, ncar, inv, kB.lin, kB.k, CB);
  }
  for (int c = 0; c < nce; ++c)
    ceff[(long)c * g.Mhalf + i] = to_v<V>(make_double2(CA[c].x + CB[c].x, CA[c].y - CB[c].y));
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
  k_ceff<typename Vec2<T>::t><<<nblk(g.Mhalf, 256), 256, 0, st>>>(g, kt, carrier, in_f64, comp_stride, ncomp_carrier,
                                                                 invariant, two_thirds, shell_full, ceff, nceff, seff);
  fit_prof_end(st);
  FIT_LAUNCH_CHECK();
  return FIT_OK;
}

// ---- shell binning ----------------------------------------------------------------------------
// Block-local FP64 bins in shared memory (lanes with the same shell are combined with warp
// shuffles first), per-block partials, then a fixed-order reduction over blocks.

template <typename V>
__global__ void k_bin(const V* __restrict__ nh, long bstride, int nb, const V* __restrict__ ceff, int nc,
                      const uint16_t* __restrict__ seff, long Mhalf, int nsh, double* __restrict__ partial) {
  extern __shared__ double bins[];
  const int nbins = nb * nsh;
  for (int t = threadIdx.x; t < nbins; t += blockDim.x) bins[t] = 0.0;
  __syncthreads();
  const long step = (long)gridDim.x * blockDim.x;
  const long iters = (Mhalf + step - 1) / step;
  const unsigned lane = threadIdx.x & 31;
  for (long it = 0; it < iters; ++it) {
    const long i = it * step + blockIdx.x * (long)blockDim.x + threadIdx.x;
    int s = 0;
    V cf[3];
    if (i < Mhalf) {
      s = seff[i];
      if (s) for (int c = 0; c < nc; ++c) cf[c] = ceff[(long)c * Mhalf + i];
    }
    const unsigned grp = __match_any_sync(0xffffffffu, s);
    const int leader = __ffs(grp) - 1;
    for (int b = 0; b < nb; ++b) {
      double v = 0.0;
      if (s) {
        for (int c = 0; c < nc; ++c) {
          const V x = nh[b * bstride + (long)c * Mhalf + i];
          v += (double)cf[c].x * (double)x.x + (double)cf[c].y * (double)x.y;
        }
      }
      double sum = 0.0;
      for (unsigned m = grp; m; m &= m - 1) sum += __shfl_sync(grp, v, __ffs(m) - 1);
      if (s && (int)lane == leader) atomicAdd(&bins[b * nsh + (s - 1)], sum);
    }
  }
  __syncthreads();
  for (int t = threadIdx.x; t < nbins; t += blockDim.x) partial[(long)blockIdx.x * nbins + t] = bins[t];
}

__global__ void k_reduce_partials(const double* __restrict__ partial, int nblocks, int nbins, double* out) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= nbins) return;
  double s = 0.0;
  for (int b = 0; b < nblocks; ++b) s += partial[(long)b * nbins + j];
  out[j] = s;
}

template <typename T>
int bin_density(const GridDesc& g, const typename Vec2<T>::t* nh, long nh_batch_stride, int nb,
                const typename Vec2<T>::t* ceff, int nc, const uint16_t* seff, int nsh, double* partial,
                long partial_cap, double* out, cudaStream_t st) {
  const int nbins = nb * nsh;
  const size_t smem = sizeof(double) * nbins;
  if (smem > 96 * 1024) {
    fit_set_error("too many shell bins (%d) for one binning launch", nbins);
    return FIT_ERR_SIZE;
  }
  int nblocks = 2 * 152;
  const long needed = (g.Mhalf + 255) / 256;
  if (needed < nblocks) nblocks = (int)needed;
  if ((long)nblocks * nbins > partial_cap) nblocks = (int)(partial_cap / nbins);
  if (nblocks < 1) {
    fit_set_error("binning scratch too small");
    return FIT_ERR_SIZE;
  }
  if (smem > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(k_bin<typename Vec2<T>::t>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem);
    if (e != cudaSuccess) {
      fit_set_error("cudaFuncSetAttribute failed: %s", cudaGetErrorString(e));
      return FIT_ERR_CUDA;
    }
  }
  fit_prof_begin(PK_BIN, (double)g.Mhalf * ((nb + 1) * nc * sizeof(typename Vec2<T>::t) + 2.0), st);
  k_bin<typename Vec2<T>::t><<<nblocks, 256, smem, st>>>(nh, nh_batch_stride, nb, ceff, nc, seff, g.Mhalf, nsh,
                                                        partial);
  fit_prof_end(st);
  FIT_LAUNCH_CHECK();
  k_reduce_partials<<<nblk(nbins, 128), 128, 0, st>>>(partial, nblocks, nbins, out);
  FIT_LAUNCH_CHECK();
  return FIT_OK;
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
__global__ void k_helical(GridDesc g, KTab kt, const void* u, int f64, void* up, void* um) {
  const long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (i >= g.Ntot) return;
  int k[3];
  k[0] = (int)(i % g.N[0]);
  const long r = i / g.N[0];
  k[1] = (int)(r % g.N[1]);
  k[2] = (int)(r / g.N[1]);
  const double kx = kt.k[0][k[0]], ky = kt.k[1][k[1]], kz = kt.k[2][k[2]];
  const double kk = sqrt(kx * kx + ky * ky + kz * kz);
  const long n = g.Ntot;
  if (kk == 0.0) {
    for (int c = 0; c < 3; ++c) {
      st_c(up, f64, i + n * c, make_double2(0, 0));
      st_c(um, f64, i + n * c, make_double2(0, 0));
    }
    return;
  }
  const double hx = kx / kk, hy = ky / kk, hz = kz / kk;
  double rx = 0, ry = 0, rz = 1;
  if (!(fabs(hz) < 0.9)) { rx = 1; rz = 0; }
  double e1x = hy * rz - hz * ry, e1y = hz * rx - hx * rz, e1z = hx * ry - hy * rx;
  const double n1 = sqrt(e1x * e1x + e1y * e1y + e1z * e1z);
  e1x /= n1; e1y /= n1; e1z /= n1;
  const double e2x = hy * e1z - hz * e1y, e2y = hz * e1x - hx * e1z, e2z = hx * e1y - hy * e1x;
  const double2 u1 = ld_c(u, f64, i), u2 = ld_c(u, f64, i + n), u3 = ld_c(u, f64, i + 2 * n);
  const double2 ue1 = make_double2(u1.x * e1x + u2.x * e1y + u3.x * e1z, u1.y * e1x + u2.y * e1y + u3.y * e1z);
  const double2 ue2 = make_double2(u1.x * e2x + u2.x * e2y + u3.x * e2z, u1.y * e2x + u2.y * e2y + u3.y * e2z);
  const double is2 = 1.0 / sqrt(2.0);
  // u+ coefficient (ue1 - i ue2)/sqrt2, u- coefficient (ue1 + i ue2)/sqrt2
  const double2 upc = make_double2((ue1.x + ue2.y) * is2, (ue1.y - ue2.x) * is2);
  const double2 umc = make_double2((ue1.x - ue2.y) * is2, (ue1.y + ue2.x) * is2);
  const double e1[3] = {e1x, e1y, e1z}, e2[3] = {e2x, e2y, e2z};
  for (int c = 0; c < 3; ++c) {
    const double2 hp = make_double2(e1[c] * is2, e2[c] * is2);    // (e1 + i e2)/sqrt2
    const double2 hm = make_double2(e1[c] * is2, -e2[c] * is2);   // (e1 - i e2)/sqrt2
    st_c(up, f64, i + n * c, make_double2(upc.x * hp.x - upc.y * hp.y, upc.x * hp.y + upc.y * hp.x));
    st_c(um, f64, i + n * c, make_double2(umc.x * hm.x - umc.y * hm.y, umc.x * hm.y + umc.y * hm.x));
  }
}

int helical_split(const GridDesc& g, const KTab& kt, const void* u, int in_f64, void* up, void* um, cudaStream_t st) {
  if (g.nd != 3) {
    fit_set_error("HelicalDecomposition is defined in 3D only (got nd=%d).", g.nd);
    return FIT_ERR_ARG;
  }
  k_helical<<<nblk(g.Ntot, 256), 256, 0, st>>>(g, kt, u, in_f64, up, um);
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
template int bin_density<float>(const GridDesc&, const float2*, long, int, const float2*, int, const uint16_t*, int,
                                double*, long, double*, cudaStream_t);
template int bin_density<double>(const GridDesc&, const double2*, long, int, const double2*, int, const uint16_t*,
                                 int, double*, long, double*, cudaStream_t);
template int scatter_full<float>(const GridDesc&, const float2*, int, int, void*, int, cudaStream_t);
template int scatter_full<double>(const GridDesc&, const double2*, int, int, void*, int, cudaStream_t);

}  // namespace fit
