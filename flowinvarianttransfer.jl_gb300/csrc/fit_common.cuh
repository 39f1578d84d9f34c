// Shared definitions for libfit_gb300: complex helpers, error plumbing, launch bookkeeping.
//
// Conventions (same as FlowInvariantTransfer.jl, src/Workspaces.jl:46-75):
//   * user arrays are column-major (ns..., comp), interleaved complex (ComplexF64 / ComplexF32);
//   * wavenumbers are FFTW-order with +N/2 at the Nyquist index (src/Utils.jl:51-63).
// Internally every transform runs on a half spectrum along x (kx in [0, M0/2]) of the transform
// grid M (M = N, or the 3/2-padded grid). A half-spectrum field is stored (Mh0, M1, M2)
// column-major, Mh0 = M0/2 + 1; a physical field is (M0, M1, M2) real.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <string>
#include <type_traits>

#define FIT_OK 0
#define FIT_ERR_ARG -1
#define FIT_ERR_SIZE -2
#define FIT_ERR_CUDA -3
#define FIT_ERR_ALLOC -4
#define FIT_ERR_STATE -5

#define FIT_HD __host__ __device__ __forceinline__
#define FIT_D __device__ __forceinline__

template <typename T> struct Vec2;
template <> struct Vec2<float> { typedef float2 t; };
template <> struct Vec2<double> { typedef double2 t; };

template <typename V> struct Scal;
template <> struct Scal<float2> { typedef float t; };
template <> struct Scal<double2> { typedef double t; };

template <typename V> FIT_HD V mkc(typename Scal<V>::t x, typename Scal<V>::t y) { V r; r.x = x; r.y = y; return r; }
// FP32 complex sums on the paired FP32 pipe of compute capability 10.x (one instruction for both
// parts): a + b as a paired add, a - b as the paired fma(b, -1, a), which rounds once like the
// scalar subtraction (b * -1 is exact). Each is the scalar operation bit for bit, but the compiler
// no longer fuses a preceding product into the sum, so transforms differ at FP32 rounding level.
template <typename V> FIT_HD V cadd(V a, V b) {
#if defined(__CUDA_ARCH__) && __CUDA_ARCH__ >= 1000
  if constexpr (std::is_same<V, float2>::value) return __fadd2_rn(a, b);
#endif
  return mkc<V>(a.x + b.x, a.y + b.y);
}
template <typename V> FIT_HD V csub(V a, V b) {
#if defined(__CUDA_ARCH__) && __CUDA_ARCH__ >= 1000
  if constexpr (std::is_same<V, float2>::value) return __ffma2_rn(b, make_float2(-1.f, -1.f), a);
#endif
  return mkc<V>(a.x - b.x, a.y - b.y);
}
template <typename V> FIT_HD V cmul(V a, V b) { return mkc<V>(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x); }
template <typename V> FIT_HD V cconj(V a) { return mkc<V>(a.x, -a.y); }
template <typename V, typename S> FIT_HD V cscale(V a, S s) { return mkc<V>(a.x * s, a.y * s); }
// multiply by +i (POS) or -i
template <typename V, bool POS> FIT_HD V cmuli(V a) { return POS ? mkc<V>(-a.y, a.x) : mkc<V>(a.y, -a.x); }

// Thread-local error string for fit_last_error().
void fit_set_error(const char* fmt, ...);
const char* fit_get_error();

// Clock bound of every wait on a bulk copy or a tensor-core commit inside a kernel (about 1 s at
// 2 GHz); bounds below FIT_WAIT_POLL_MIN poll without suspending (fit_tma.cuh).
#define FIT_WAIT_CYCLES 2000000000LL
#define FIT_WAIT_POLL_MIN 4096LL
// Bound passed to the kernels' first waits: FIT_WAIT_CYCLES, or the value of the environment
// variable FIT_TEST_WAIT_CYCLES when it is set to a positive number. Tests set it to a few cycles
// so that the waits run out and the error path (device flag -> host error code) is exercised with
// copies and commits that still complete; it is read at every launch (graphs keep the value they
// were captured with).
long long fit_wait_cycles();

// Every launch of a library kernel is counted (graph replays add the kernels they contain).
void fit_count_launches(long n);
long fit_launch_total();

#define FIT_CUDA_CHECK(expr)                                                                 \
  do {                                                                                     \
    cudaError_t _e = (expr);                                                               \
    if (_e != cudaSuccess) {                                                               \
      fit_set_error("%s failed: %s (%s:%d)", #expr, cudaGetErrorString(_e), __FILE__, __LINE__); \
      return FIT_ERR_CUDA;                                                                 \
    }                                                                                      \
  } while (0)

#define FIT_LAUNCH_CHECK()                                                                   \
  do {                                                                                     \
    cudaError_t _e = cudaGetLastError();                                                   \
    if (_e != cudaSuccess) {                                                               \
      fit_set_error("kernel launch failed: %s (%s:%d)", cudaGetErrorString(_e), __FILE__, __LINE__); \
      return FIT_ERR_CUDA;                                                                 \
    }                                                                                      \
    fit_count_launches(1);                                                                 \
  } while (0)

#define FIT_TRY(expr)            \
  do {                           \
    int _rc = (expr);            \
    if (_rc != FIT_OK) return _rc; \
  } while (0)

// Optional per-launch timing (CUDA events around each launch, eager launches only) with the
// launch's algorithmic DRAM bytes; read back through fit_prof_read().
enum ProfKind {
  PK_FFT_STRIDED = 0, PK_FFT_C2R_X, PK_FFT_R2C_X, PK_GATHER, PK_PRODUCT, PK_BIN, PK_CARRIER, PK_TRIAD,
  PK_SHELL, PK_S2S_ZINV, PK_S2S_YINV, PK_S2S_XMIX, PK_S2S_YFWD, PK_S2S_ZFWD_BIN, PK_S2S_VELOCITY, PK_FFT_Z_FULL,
  PK_COUNT
};
bool fit_prof_on();
void fit_prof_begin(int kind, double bytes, cudaStream_t st);
void fit_prof_end(cudaStream_t st);

// Shared-memory carveout sized for occupancy: the blocks per SM that threads and registers allow,
// times the block's shared footprint (+1 KB reserved per block), as a percentage of the SM's 228 KB;
// the rest stays L1. (Leaving the default can cap resident blocks; asking for the maximum shrinks L1
// for kernels that do not need it.)
template <typename K>
inline cudaError_t set_occupancy_carveout(K kern, size_t dyn_smem, int nthr) {
  cudaFuncAttributes fa;
  cudaError_t e = cudaFuncGetAttributes(&fa, kern);
  if (e != cudaSuccess) return e;
  const int regs = fa.numRegs > 0 ? ((fa.numRegs + 7) / 8) * 8 : 32;
  int blocks = 2048 / (nthr > 0 ? nthr : 1);
  const int by_regs = 65536 / (regs * (nthr > 0 ? nthr : 1));
  if (by_regs < blocks) blocks = by_regs;
  if (blocks < 1) blocks = 1;
  const double need = (double)blocks * ((double)dyn_smem + (double)fa.sharedSizeBytes + 1024.0);
  int pct = (int)(100.0 * need / (228.0 * 1024.0) + 0.999);
  if (pct > 100) pct = 100;
  if (pct < 0) pct = 0;
  return cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout, pct);
}

// Radix schedule of one transform length (product of the entries = N).
struct Radices {
  int n;
  int r[16];
};

// Geometry of the transform grid and its relation to the user grid.
//   N: user (data) grid; M: transform grid (M == N unless padded); Mh0 = M0/2 + 1.
struct GridDesc {
  int nd;
  int N[3];
  int M[3];
  int Mh0;
  int padded;     // 1 for the 3/2 path
  long Ntot;      // prod N
  long Mtot;      // prod M (physical points)
  long Mhalf;     // Mh0 * M1 * M2 (half-spectrum modes)
};
