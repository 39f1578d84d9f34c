// Resolved mode-to-mode transfer S(k|p) as a direct triad evaluation.
//
// calculate_mode_to_mode_transfer (src/ScaleToScale/ScaleToScaleTransfer.jl:49-91) runs one full
// nonlinear term per giver mode p with the advected field restricted to p. Writing that
// nonlinear term (_nonlinear_term_fft!, ext/FlowInvariantTransferFFTWExt.jl:61-121) for a
// single-mode field in closed form gives, for every receiver k,
//   N_p,c(k) = keep(k)/(2 Np^2) * sum_j [ A_j(k-p) i k_j(p) f_c(p) + A_j(k+p) conj(i k_j(p) f_c(p)) ]
// with A = Herm(keep * u_adv) (what real(ifft) keeps of the advecting velocity), f = keep * u,
// and k -/+ p taken mod N (the FFT's aliasing wrap). Then
//   S(k|p) = sum_c Re(conj(C_c(k)) N_p,c(k)),  C = the invariant's effective carrier.
// One thread owns one receiver k and sweeps a chunk of givers p, writing the column-major
// S[k + Nm p] (coalesced across the warp) and accumulating net(k) in FP64.
#include "fit_plan.cuh"

namespace fit {

struct TriadArgs {
  int nd, N[3];
  long Nm;
  int two_thirds;
  double norm;   // 1/(2 Nm^2)
};

FIT_D bool keep_k(const TriadArgs& t, const int* k) {
  if (!t.two_thirds) return true;
  for (int d = 0; d < t.nd; ++d) {
    const int N = t.N[d];
    const int a = (k[d] <= N / 2) ? k[d] : N - k[d];
    if (a >= N / 3) return false;
  }
  return true;
}

// Precompute A (nd comps), f (M comps) and the effective carrier C (M comps) on the full grid.
template <typename V>
__global__ void k_triad_prep(GridDesc g, KTab kt, TriadArgs t, const void* u, const void* adv, int f64, int M,
                             int inv, V* A, V* F, V* C) {
  const long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (i >= t.Nm) return;
  int k[3], kn[3];
  k[0] = (int)(i % t.N[0]);
  const long r = i / t.N[0];
  k[1] = (int)(r % t.N[1]);
  k[2] = (int)(r / t.N[1]);
  for (int d = 0; d < 3; ++d) kn[d] = (t.N[d] - k[d]) % t.N[d];
  const long ineg = kn[0] + (long)t.N[0] * (kn[1] + (long)t.N[1] * kn[2]);
  const bool kp = keep_k(t, k);
  for (int j = 0; j < t.nd; ++j) {
    double2 a = make_double2(0, 0);
    if (kp) {
      const double2 x = f64 ? ((const double2*)adv)[i + t.Nm * j] : make_double2(((const float2*)adv)[i + t.Nm * j].x, ((const float2*)adv)[i + t.Nm * j].y);
      const double2 y = f64 ? ((const double2*)adv)[ineg + t.Nm * j] : make_double2(((const float2*)adv)[ineg + t.Nm * j].x, ((const float2*)adv)[ineg + t.Nm * j].y);
      a = make_double2(0.5 * (x.x + y.x), 0.5 * (x.y - y.y));
    }
    V av; av.x = a.x; av.y = a.y;
    A[i + t.Nm * j] = av;
  }
  double2 cc[3];
  // effective carrier from the untruncated field
  {
    double2 uu[3];
    for (int c = 0; c < M; ++c)
      uu[c] = f64 ? ((const double2*)u)[i + t.Nm * c] : make_double2(((const float2*)u)[i + t.Nm * c].x, ((const float2*)u)[i + t.Nm * c].y);
    if (inv == INV_KE || inv == INV_SCALAR) {
      for (int c = 0; c < M; ++c) cc[c] = uu[c];
    } else {
      const double kx = kt.k[0][k[0]];
      const double ky = t.nd >= 2 ? kt.k[1][k[1]] : 0.0;
      const double kz = t.nd >= 3 ? kt.k[2][k[2]] : 0.0;
      if (inv == INV_ENSTROPHY && t.nd == 2) {
        const double2 w = make_double2(-(kx * uu[1].y - ky * uu[0].y), kx * uu[1].x - ky * uu[0].x);
        cc[0] = make_double2(-w.y * ky, w.x * ky);
        cc[1] = make_double2(w.y * kx, -w.x * kx);
      } else {
        double2 w[3];
        w[0] = make_double2(-(ky * uu[2].y - kz * uu[1].y), ky * uu[2].x - kz * uu[1].x);
        w[1] = make_double2(-(kz * uu[0].y - kx * uu[2].y), kz * uu[0].x - kx * uu[2].x);
        w[2] = make_double2(-(kx * uu[1].y - ky * uu[0].y), kx * uu[1].x - ky * uu[0].x);
        if (inv == INV_HELICITY) {
          cc[0] = w[0]; cc[1] = w[1]; cc[2] = w[2];
        } else {
          cc[0] = make_double2(-(ky * w[2].y - kz * w[1].y), ky * w[2].x - kz * w[1].x);
          cc[1] = make_double2(-(kz * w[0].y - kx * w[2].y), kz * w[0].x - kx * w[2].x);
          cc[2] = make_double2(-(kx * w[1].y - ky * w[0].y), kx * w[1].x - ky * w[0].x);
        }
      }
    }
    for (int c = 0; c < M; ++c) {
      V fv, cv;
      fv.x = kp ? uu[c].x : 0.0;
      fv.y = kp ? uu[c].y : 0.0;
      cv.x = cc[c].x;
      cv.y = cc[c].y;
      F[i + t.Nm * c] = fv;
      C[i + t.Nm * c] = cv;
    }
  }
}

template <typename V, int M, int ND>
__global__ void __launch_bounds__(256) k_triad(TriadArgs t, KTab kt, const V* __restrict__ A, const V* __restrict__ F,
                                               const V* __restrict__ Cc, long pchunk, double* __restrict__ S,
                                               double* __restrict__ netpart) {
  typedef typename Scal<V>::t R;
  const long k = blockIdx.x * (long)blockDim.x + threadIdx.x;
  const long p0 = blockIdx.y * pchunk;
  long p1 = p0 + pchunk;
  if (p1 > t.Nm) p1 = t.Nm;
  if (k >= t.Nm) return;
  int kk[3];
  kk[0] = (int)(k % t.N[0]);
  const long r = k / t.N[0];
  kk[1] = (int)(r % t.N[1]);
  kk[2] = (int)(r / t.N[1]);
  const bool kp = keep_k(t, kk);
  double net = 0.0;
  if (!kp) {
    for (long p = p0; p < p1; ++p) S[k + t.Nm * p] = 0.0;
    netpart[blockIdx.y * t.Nm + k] = 0.0;
    return;
  }
  V ck[M];
#pragma unroll
  for (int c = 0; c < M; ++c) ck[c] = Cc[k + t.Nm * c];
  int pp[3];
  pp[0] = (int)(p0 % t.N[0]);
  const long rp = p0 / t.N[0];
  pp[1] = (int)(rp % t.N[1]);
  pp[2] = (int)(rp / t.N[1]);
  const R norm = (R)t.norm;
  for (long p = p0; p < p1; ++p) {
    V fp[M];
    bool nz = false;
#pragma unroll
    for (int c = 0; c < M; ++c) {
      fp[c] = F[p + t.Nm * c];
      nz |= (fp[c].x != (R)0) || (fp[c].y != (R)0);
    }
    double sv = 0.0;
    if (nz) {
      long im = 0, ip = 0, st = 1;
#pragma unroll
      for (int d = 0; d < ND; ++d) {
        int a = kk[d] - pp[d];
        if (a < 0) a += t.N[d];
        int b = kk[d] + pp[d];
        if (b >= t.N[d]) b -= t.N[d];
        im += a * st;
        ip += b * st;
        st *= t.N[d];
      }
      V a1 = mkc<V>(0, 0), a2 = mkc<V>(0, 0);
#pragma unroll
      for (int j = 0; j < ND; ++j) {
        const R kj = (R)kt.k[j][pp[j]];
        const V x = A[im + t.Nm * j], y = A[ip + t.Nm * j];
        a1.x += x.x * kj; a1.y += x.y * kj;
        a2.x += y.x * kj; a2.y += y.y * kj;
      }
      V cf = mkc<V>(0, 0), cfc = mkc<V>(0, 0);
#pragma unroll
      for (int c = 0; c < M; ++c) {
        // conj(ck) * fp and conj(ck) * conj(fp)
        cf.x += ck[c].x * fp[c].x + ck[c].y * fp[c].y;
        cf.y += ck[c].x * fp[c].y - ck[c].y * fp[c].x;
        cfc.x += ck[c].x * fp[c].x - ck[c].y * fp[c].y;
        cfc.y += -ck[c].x * fp[c].y - ck[c].y * fp[c].x;
      }
      // Re(i a1 cf - i a2 cfc) = -Im(a1 cf) + Im(a2 cfc)
      const R im1 = a1.x * cf.y + a1.y * cf.x;
      const R im2 = a2.x * cfc.y + a2.y * cfc.x;
      sv = (double)((im2 - im1) * norm);
    }
    S[k + t.Nm * p] = sv;
    net += sv;
    if (++pp[0] == t.N[0]) {
      pp[0] = 0;
      if (++pp[1] == t.N[1]) {
        pp[1] = 0;
        ++pp[2];
      }
    }
  }
  netpart[blockIdx.y * t.Nm + k] = net;
}

__global__ void k_triad_net(const double* __restrict__ part, int nchunk, long Nm, double* net) {
  const long k = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (k >= Nm) return;
  double s = 0.0;
  for (int c = 0; c < nchunk; ++c) s += part[c * Nm + k];
  net[k] = s;
}

template <typename V, int M>
static void launch_triad(dim3 grid, const TriadArgs& t, const KTab& kt, const V* A, const V* F, const V* C, long pch,
                         double* S, double* np, cudaStream_t st) {
  if (t.nd == 1) k_triad<V, M, 1><<<grid, 256, 0, st>>>(t, kt, A, F, C, pch, S, np);
  else if (t.nd == 2) k_triad<V, M, 2><<<grid, 256, 0, st>>>(t, kt, A, F, C, pch, S, np);
  else k_triad<V, M, 3><<<grid, 256, 0, st>>>(t, kt, A, F, C, pch, S, np);
}

template <typename V>
static int triad_run(fit_plan* p, const void* u, const void* adv, int inv, double* S, double* net) {
  TriadArgs t;
  t.nd = p->nd;
  for (int d = 0; d < 3; ++d) t.N[d] = p->g.N[d];
  t.Nm = p->g.Ntot;
  t.two_thirds = p->dealias == 1;
  t.norm = 0.5 / ((double)t.Nm * (double)t.Nm);
  const int M = p->M;
  const int nchunk = 16;
  const long pch = (t.Nm + nchunk - 1) / nchunk;
  FIT_TRY(ensure(p, &p->hs, sizeof(V) * (size_t)t.Nm * (p->nd + 2 * M) + sizeof(double) * nchunk * t.Nm));
  V* A = (V*)p->hs.p;
  V* F = A + t.Nm * p->nd;
  V* C = F + t.Nm * M;
  double* part = (double*)(C + t.Nm * M);
  const unsigned nb = (unsigned)((t.Nm + 255) / 256);
  k_triad_prep<V><<<nb, 256, 0, p->stream>>>(p->g, p->kt, t, u, adv, p->io_f64, M, inv, A, F, C);
  FIT_LAUNCH_CHECK();
  dim3 grid(nb, nchunk);
  fit_prof_begin(PK_TRIAD, 8.0 * (double)t.Nm * (double)t.Nm, p->stream);
  if (M == 1) launch_triad<V, 1>(grid, t, p->kt, A, F, C, pch, S, part, p->stream);
  else if (M == 2) launch_triad<V, 2>(grid, t, p->kt, A, F, C, pch, S, part, p->stream);
  else launch_triad<V, 3>(grid, t, p->kt, A, F, C, pch, S, part, p->stream);
  fit_prof_end(p->stream);
  FIT_LAUNCH_CHECK();
  k_triad_net<<<nb, 256, 0, p->stream>>>(part, nchunk, t.Nm, net);
  FIT_LAUNCH_CHECK();
  return FIT_OK;
}

int triad_m2m(fit_plan* p, const void* u, const void* adv, int inv, int fp64, double* S, double* net) {
  if (fp64) return triad_run<double2>(p, u, adv, inv, S, net);
  return triad_run<float2>(p, u, adv, inv, S, net);
}

}  // namespace fit

namespace fit {

// Same three launches as triad_run, with the A/F/C tables and the per-chunk net partials placed
// in caller-provided scratch (used by the allocation-free entry point in fit_noalloc.cu).
int triad_run_scratch(const GridDesc& g, const KTab& kt, int M, int two_thirds, int io_f64, const void* u,
                      const void* adv, int inv, int fp64, void* scratch, int nchunk, double* S, double* net,
                      cudaStream_t st) {
  TriadArgs t;
  t.nd = g.nd;
  for (int d = 0; d < 3; ++d) t.N[d] = g.N[d];
  t.Nm = g.Ntot;
  t.two_thirds = two_thirds;
  t.norm = 0.5 / ((double)t.Nm * (double)t.Nm);
  const long pch = (t.Nm + nchunk - 1) / nchunk;
  const unsigned nb = (unsigned)((t.Nm + 255) / 256);
  dim3 grid(nb, nchunk);
  if (fp64) {
    double2* A = (double2*)scratch;
    double2* F = A + t.Nm * t.nd;
    double2* C = F + t.Nm * M;
    double* part = (double*)(C + t.Nm * M);
    k_triad_prep<double2><<<nb, 256, 0, st>>>(g, kt, t, u, adv, io_f64, M, inv, A, F, C);
    FIT_LAUNCH_CHECK();
    if (M == 1) launch_triad<double2, 1>(grid, t, kt, A, F, C, pch, S, part, st);
    else if (M == 2) launch_triad<double2, 2>(grid, t, kt, A, F, C, pch, S, part, st);
    else launch_triad<double2, 3>(grid, t, kt, A, F, C, pch, S, part, st);
    FIT_LAUNCH_CHECK();
    k_triad_net<<<nb, 256, 0, st>>>(part, nchunk, t.Nm, net);
  } else {
    float2* A = (float2*)scratch;
    float2* F = A + t.Nm * t.nd;
    float2* C = F + t.Nm * M;
    double* part = (double*)(C + t.Nm * M);
    k_triad_prep<float2><<<nb, 256, 0, st>>>(g, kt, t, u, adv, io_f64, M, inv, A, F, C);
    FIT_LAUNCH_CHECK();
    if (M == 1) launch_triad<float2, 1>(grid, t, kt, A, F, C, pch, S, part, st);
    else if (M == 2) launch_triad<float2, 2>(grid, t, kt, A, F, C, pch, S, part, st);
    else launch_triad<float2, 3>(grid, t, kt, A, F, C, pch, S, part, st);
    FIT_LAUNCH_CHECK();
    k_triad_net<<<nb, 256, 0, st>>>(part, nchunk, t.Nm, net);
  }
  FIT_LAUNCH_CHECK();
  return FIT_OK;
}

}  // namespace fit
