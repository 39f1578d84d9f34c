// Fused shell-to-shell kernels instantiated for cube sizes 64 128 256 512.
#include <math.h>
#include <string.h>

#include <vector>

#include "fit_fused_impl.cuh"

namespace fit {

// Returns 1 when N is not built in this translation unit.
int fz_dispatch_a(int N, const FzArgs& a, const float2* H, const float2* Ceff, const uint16_t* seff,
                    const float* kd, const float* U, float2* bufA, float2* bufB,
                    double* partial, const float2* tw, int* err, cudaStream_t st) {
  switch (N) {
    case 64: return fz_batch<64>(a, H, Ceff, seff, kd, U, bufA, bufB, partial, tw, err, st);
    case 128: return fz_batch<128>(a, H, Ceff, seff, kd, U, bufA, bufB, partial, tw, err, st);
    case 256: return fz_batch<256>(a, H, Ceff, seff, kd, U, bufA, bufB, partial, tw, err, st);
    case 512: return fz_batch<512>(a, H, Ceff, seff, kd, U, bufA, bufB, partial, tw, err, st);
    default: return 1;
  }
}

// zinv of a batch over pencil tiles [t0, t1) (1 when N is not built here).
int fz_zinv_a(int N, const FzArgs& a, const float2* H, const float* kd, float2* bufA, const float2* tw, int t0,
               int t1, cudaStream_t st) {
  switch (N) {
    case 64: return fz_zinv_tiles<64>(a, H, kd, bufA, tw, t0, t1, st);
    case 128: return fz_zinv_tiles<128>(a, H, kd, bufA, tw, t0, t1, st);
    case 256: return fz_zinv_tiles<256>(a, H, kd, bufA, tw, t0, t1, st);
    case 512: return fz_zinv_tiles<512>(a, H, kd, bufA, tw, t0, t1, st);
    default: return 1;
  }
}

// Pencils per tile of the fused strided passes for transform length N (0 when not built here).
int fz_tile_cols_a(int N) {
  switch (N) {
    case 64: return FzTile<64>::C;
    case 128: return FzTile<128>::C;
    case 256: return FzTile<256>::C;
    case 512: return FzTile<512>::C;
    default: return 0;
  }
}

// Self-advecting velocity in physical space over the live box (1 when N is not built here).
int fz_velocity_a(int N, const FzArgs& a, const float2* H, float2* bufZ, float2* bufY, float* U, const float2* tw,
                   float scale, cudaStream_t st) {
  switch (N) {
    case 64: return fz_velocity<64>(a, H, bufZ, bufY, U, tw, scale, st);
    case 128: return fz_velocity<128>(a, H, bufZ, bufY, U, tw, scale, st);
    case 256: return fz_velocity<256>(a, H, bufZ, bufY, U, tw, scale, st);
    case 512: return fz_velocity<512>(a, H, bufZ, bufY, U, tw, scale, st);
    default: return 1;
  }
}

// Whole-box nonlinear terms of a batch (1 when N is not built here).
int fz_terms_a(int N, const FzArgs& a, const float2* H, const float* kd, const float* U, float2* bufA, float2* bufB,
               float2* Nout, const float2* tw, int* err, cudaStream_t st) {
  switch (N) {
    case 64: return fz_terms<64>(a, H, kd, U, bufA, bufB, Nout, tw, err, st);
    case 128: return fz_terms<128>(a, H, kd, U, bufA, bufB, Nout, tw, err, st);
    case 256: return fz_terms<256>(a, H, kd, U, bufA, bufB, Nout, tw, err, st);
    case 512: return fz_terms<512>(a, H, kd, U, bufA, bufB, Nout, tw, err, st);
    default: return 1;
  }
}

}  // namespace fit

// ---- benchmark hook: one fused pass alone on synthetic device data ----------------------------------
namespace {

__global__ void k_bench_fill(float* p, long n, unsigned seed) {
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
    unsigned h = (unsigned)i * 2654435761u ^ seed;
    h ^= h >> 13;
    h *= 0x5bd1e995u;
    h ^= h >> 15;
    p[i] = (float)(h & 0xffffff) / 16777216.0f - 0.5f;
  }
}

// shell index of live-box mode (kx, f_y, f_z) in shells of width dk (0 beyond the last shell)
__global__ void k_bench_shells(uint16_t* seff, int K, int KX, long P1, long P1S, float dk, int nsh) {
  const long n = (long)(2 * K + 1) * P1S;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
    const long col = i % P1S;
    if (col >= P1) {   // row padding
      seff[i] = 0;
      continue;
    }
    const int kx = (int)(col % KX), fy = (int)(col / KX) - K, fz = (int)(i / P1S) - K;
    const int sh = (int)(sqrtf((float)(kx * kx + fy * fy + fz * fz)) / dk) + 1;
    seff[i] = (uint16_t)(sh <= nsh ? sh : 0);
  }
}

template <int N>
int bench_pass(int pass, long units, int reps, double* ms, double* bytes) {
  using namespace fit;
  const int K = N / 3 - 1, KX = K + 1, KY = 2 * K + 1;
  const long P1 = (long)KX * KY, L = (long)N * N;
  FzArgs a;
  memset(&a, 0, sizeof(a));
  a.K = K;
  a.KX = KX;
  a.KY = KY;
  a.P1 = P1;
  fz_set_strides(&a);
  a.L = pass == 0 ? units : L;
  a.nsh = pass == 2 ? 32 : 1;
  a.nb = pass == 2 ? (int)units : 1;
  for (int b = 0; b < a.nb; ++b) {
    a.med[b] = b + 1;
    a.ext[b][0] = a.ext[b][1] = a.ext[b][2] = (short)K;
  }
  a.so = 1.0f / ((float)N * N * N);
  const long Mtot = (long)N * N * N;
  // pass 0 (x pass): G (9 lines x KX per line), U (3 velocity fields, the last one sliced), out (3 x KX);
  // pass 1 (y inverse): the six z-pass outputs of all N planes in, nine y-pass outputs out;
  // pass 2 (z forward + binning, `units` mediators): their y-forward outputs in (3 x N x P1 each),
  // the effective carrier (3 x KY x P1, in U's place) and shell ids of 32 shells of width 14 N/512,
  // block partials out
  const long pt = (P1 + FzTile<N>::C - 1) / FzTile<N>::C;
  const size_t in_n = pass == 0 ? (size_t)9 * units * a.KXS : pass == 1 ? (size_t)6 * N * a.P1S
                                                                         : (size_t)3 * units * N * a.P1S;
  const size_t un = pass == 0 ? (size_t)(2 * Mtot + units * (long)N) : pass == 1 ? (size_t)KY : (size_t)6 * KY * a.P1S;
  const size_t on = pass == 0 ? (size_t)3 * units * a.KXS : pass == 1 ? (size_t)9 * L * a.KXS : (size_t)units * 32 * pt;
  uint16_t* seff = nullptr;
  float2 *in = nullptr, *out = nullptr, *tw = nullptr;
  float* U = nullptr;
  int* err = nullptr;
  cudaStream_t st = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  int rc = FIT_OK;
  std::vector<float2> h(N);
  for (int t = 0; t < N; ++t) {
    const long double ang = -2.0L * 3.14159265358979323846264338327950288L * t / N;
    h[t] = make_float2((float)cosl(ang), (float)sinl(ang));
  }
  auto ck = [&](cudaError_t e) {
    if (e != cudaSuccess && rc == FIT_OK) {
      fit_set_error("fused-pass benchmark: %s", cudaGetErrorString(e));
      rc = FIT_ERR_CUDA;
    }
    return rc == FIT_OK;
  };
  auto launch = [&]() -> int {
    if (pass == 0) return fz_xpass<N>(a, in, U, out, tw, err, st);
    if (pass == 1) return fz_yinv<N>(a, in, U, out, tw, err, (int)units, st);
    return fz_zfwd_bin<N>(a, in, (const float2*)U, seff, (double*)out, tw, st);
  };
  if (ck(cudaMalloc(&in, in_n * 8)) && ck(cudaMalloc(&U, un * 4)) && ck(cudaMalloc(&out, on * 8)) &&
      ck(cudaMalloc(&seff, (pass == 2 ? (size_t)KY * a.P1S : 1) * sizeof(uint16_t))) &&
      ck(cudaMalloc(&tw, (size_t)N * 8)) && ck(cudaMalloc(&err, sizeof(int))) && ck(cudaStreamCreate(&st)) &&
      ck(cudaEventCreate(&e0)) && ck(cudaEventCreate(&e1)) && ck(cudaMemsetAsync(err, 0, sizeof(int), st)) &&
      ck(cudaMemcpyAsync(tw, h.data(), (size_t)N * 8, cudaMemcpyHostToDevice, st))) {
    k_bench_fill<<<1216, 256, 0, st>>>((float*)in, (long)in_n * 2, 1u);
    k_bench_fill<<<1216, 256, 0, st>>>(U, (long)un, 2u);
    if (pass == 2) k_bench_shells<<<1216, 256, 0, st>>>(seff, K, KX, P1, a.P1S, 14.0f * N / 512.0f, 32);
    rc = launch();   // warm-up (kernel attributes)
    if (rc == FIT_OK && ck(cudaEventRecord(e0, st))) {
      for (int r = 0; r < reps && rc == FIT_OK; ++r) rc = launch();
      float t = 0.f;
      if (rc == FIT_OK && ck(cudaEventRecord(e1, st)) && ck(cudaStreamSynchronize(st)) &&
          ck(cudaEventElapsedTime(&t, e0, e1))) {
        *ms = (double)t / reps;
        *bytes = pass == 0   ? 8.0 * 12.0 * (double)units * KX + 4.0 * 3.0 * (double)N * units
                 : pass == 1 ? 8.0 * ((double)units * (6.0 * P1 + 9.0 * (double)N * KX))
                             : 8.0 * ((double)units * 3.0 * N * P1 + 3.0 * KY * P1) + 2.0 * KY * P1;
        int hf = 0;
        if (ck(cudaMemcpy(&hf, err, sizeof(int), cudaMemcpyDeviceToHost)) && hf) {
          fit_set_error("fused-pass benchmark: a bounded wait timed out");
          rc = FIT_ERR_STATE;
        }
      }
    }
  }
  if (st) cudaStreamSynchronize(st);
  cudaFree(in);
  cudaFree(U);
  cudaFree(out);
  cudaFree(tw);
  cudaFree(err);
  cudaFree(seff);
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  if (st) cudaStreamDestroy(st);
  return rc;
}

}  // namespace

extern "C" int fit_bench_fused_pass(int pass, int N, long long units, int reps, double* ms_per_launch,
                                    double* alg_bytes) {
  const long long maxu = pass == 0 ? (long long)N * N : pass == 1 ? (long long)N : 8;
  if (!ms_per_launch || !alg_bytes || reps < 1 || pass < 0 || pass > 2 || units < 1 || units > maxu ||
      (pass == 0 && units % 16 != 0)) {
    fit_set_error("fused-pass benchmark: pass 0 (x lines: a multiple of 16, at most N^2) or 1 (z planes: at "
                  "most N), reps >= 1");
    return FIT_ERR_ARG;
  }
  switch (N) {
    case 64: return bench_pass<64>(pass, units, reps, ms_per_launch, alg_bytes);
    case 128: return bench_pass<128>(pass, units, reps, ms_per_launch, alg_bytes);
    case 256: return bench_pass<256>(pass, units, reps, ms_per_launch, alg_bytes);
    case 512: return bench_pass<512>(pass, units, reps, ms_per_launch, alg_bytes);
    default:
      fit_set_error("fused-pass benchmark: transform length %d is not one of 64, 128, 256, 512", N);
      return FIT_ERR_ARG;
  }
}
