// Host launchers of the Stockham pass kernels: tile selection, twiddle tables, n-D transforms.
#include <math.h>
#include <stdlib.h>

#include <array>
#include <atomic>
#include <map>
#include <mutex>
#include <unordered_map>
#include <vector>

#include "fit_fft.cuh"
#include "fit_ops.cuh"

namespace fit {

template <typename T>
int ct_strided(const typename Vec2<T>::t* in, typename Vec2<T>::t* out, int N, long P, long Q, bool inv, T scale,
               const typename Vec2<T>::t* tw, cudaStream_t st);
template <typename T>
int ct_c2r(const typename Vec2<T>::t* in, T* out, int N, long L, T scale, const typename Vec2<T>::t* tw,
           cudaStream_t st);
template <typename T>
int ct_r2c(const T* in, typename Vec2<T>::t* out, int N, long L, T scale, const typename Vec2<T>::t* tw,
           cudaStream_t st);
template <typename T>
int ct_z_full(const typename Vec2<T>::t* in, typename Vec2<T>::t* out, int N0, int Mh0, int N1, int N2, long Q,
              const typename Vec2<T>::t* tw, cudaStream_t st);

int axis_init(Axis* a, int N) {
  a->N = N;
  a->tw32 = nullptr;
  a->tw64 = nullptr;
  if (N < 1) {
    fit_set_error("transform length %d must be positive", N);
    return FIT_ERR_SIZE;
  }
  int n = N, p2 = 0, ns = 0;
  while (n % 2 == 0) { n /= 2; ++p2; }
  int n3 = 0, n5 = 0;
  while (n % 3 == 0) { n /= 3; ++n3; }
  while (n % 5 == 0) { n /= 5; ++n5; }
  if (n != 1) {
    fit_set_error("transform length %d has a prime factor other than 2, 3, 5 (unsupported)", N);
    return FIT_ERR_SIZE;
  }
  Radices rd;
  for (int i = 0; i < p2 / 3; ++i) rd.r[ns++] = 8;
  if (p2 % 3 == 2) rd.r[ns++] = 4;
  if (p2 % 3 == 1) rd.r[ns++] = 2;
  for (int i = 0; i < n3; ++i) rd.r[ns++] = 3;
  for (int i = 0; i < n5; ++i) rd.r[ns++] = 5;
  if (ns > 16) {
    fit_set_error("transform length %d needs too many radix stages", N);
    return FIT_ERR_SIZE;
  }
  rd.n = ns;
  a->rd = rd;
  double2* h64 = (double2*)malloc(sizeof(double2) * N);
  float2* h32 = (float2*)malloc(sizeof(float2) * N);
  if (!h64 || !h32) {
    free(h64);
    free(h32);
    fit_set_error("host allocation failed");
    return FIT_ERR_ALLOC;
  }
  for (int t = 0; t < N; ++t) {
    // exact symmetric evaluation: reduce to the first octant-free form via long double
    long double ang = -2.0L * 3.14159265358979323846264338327950288L * (long double)t / (long double)N;
    double c = (double)cosl(ang), s = (double)sinl(ang);
    if (4 * t == N) { c = 0.0; s = -1.0; }
    if (2 * t == N) { c = -1.0; s = 0.0; }
    if (4 * t == 3 * N) { c = 0.0; s = 1.0; }
    h64[t] = make_double2(c, s);
    h32[t] = make_float2((float)c, (float)s);
  }
  cudaError_t e1 = cudaMalloc(&a->tw64, sizeof(double2) * N);
  cudaError_t e2 = cudaMalloc(&a->tw32, sizeof(float2) * N);
  if (e1 != cudaSuccess || e2 != cudaSuccess) {
    free(h64);
    free(h32);
    fit_set_error("cudaMalloc of twiddle tables failed");
    return FIT_ERR_ALLOC;
  }
  cudaError_t e3 = cudaMemcpy(a->tw64, h64, sizeof(double2) * N, cudaMemcpyHostToDevice);
  cudaError_t e4 = cudaMemcpy(a->tw32, h32, sizeof(float2) * N, cudaMemcpyHostToDevice);
  free(h64);
  free(h32);
  if (e3 != cudaSuccess || e4 != cudaSuccess) {
    fit_set_error("twiddle upload failed");
    return FIT_ERR_CUDA;
  }
  return FIT_OK;
}

void axis_free(Axis* a) {
  if (a->tw32) cudaFree(a->tw32);
  if (a->tw64) cudaFree(a->tw64);
  a->tw32 = nullptr;
  a->tw64 = nullptr;
}

struct Tile {
  int C, EPT, nthr;
  size_t smem;
};

// Columns per CTA: full 128-byte rows, ~64 KB of tile data (at most 128 KB), never more columns
// than exist. Elements per thread: 8 (<= 8192 elements) or 16.
static Tile pick_tile(int N, int vbytes, long avail_cols) {
  const int Cmin = 128 / vbytes;
  const long Emax = 131072 / vbytes;
  const long Etar = 65536 / vbytes;
  int C = 1;
  while ((long)C * N < Etar) C *= 2;
  if (C < Cmin) C = Cmin;
  while (C > 1 && (long)C * N > Emax) C /= 2;
  long ap2 = 1;
  while (ap2 < avail_cols) ap2 *= 2;
  if (C > ap2) C = (int)ap2;
  const long E = (long)C * N;
  Tile t;
  t.C = C;
  t.EPT = (E <= 8192) ? 8 : 16;
  long nthr = (E + t.EPT - 1) / t.EPT;
  nthr = ((nthr + 31) / 32) * 32;
  if (nthr < 32) nthr = 32;
  t.nthr = (int)nthr;
  t.smem = (size_t)(E + N) * vbytes;
  return t;
}

// Raise the dynamic shared-memory limit of a kernel once (the attribute is per function; a
// cached value keeps the call out of captured launch sequences after the first use).
template <typename K>
static int prep_kernel(K kern, size_t smem, int nthr) {
  static std::mutex mu;
  static std::unordered_map<const void*, size_t> done;
  std::lock_guard<std::mutex> lk(mu);
  auto it = done.find((const void*)kern);
  if (it != done.end() && it->second >= smem) return FIT_OK;
  cudaError_t e = cudaSuccess;
  if (smem > 48 * 1024) e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e == cudaSuccess) e = set_occupancy_carveout(kern, smem, nthr);
  if (e != cudaSuccess) {
    fit_set_error("cudaFuncSetAttribute(smem=%zu) failed: %s", smem, cudaGetErrorString(e));
    return FIT_ERR_CUDA;
  }
  done[(const void*)kern] = smem;
  return FIT_OK;
}

// ---- autotuner -------------------------------------------------------------------------------
// For each pass shape (kind, N, columns/lines, batch, element size) the first call outside a graph
// capture times every candidate kernel on scratch buffers and keeps the fastest: the compile-time
// engine (fixed tile) and the runtime engine over tile widths C (powers of two), elements per
// thread (8, 16) and radix orders (8s first, 4s first, 8s last). Later calls, captured or not,
// launch the recorded choice. Off unless enabled (fit_autotune_enable).

enum PassKind { PASS_FWD = 0, PASS_INV = 1, PASS_C2R = 2, PASS_R2C = 3 };

struct Cand {
  int engine;   // 0 compile-time kernel, 1 runtime kernel
  int C, ept, sched;
};

struct TuneEntry {
  Cand best;
  float ms_best, ms_default;
  int ncand;
};

static std::atomic<int> g_tune_on(0);
static std::mutex g_tune_mu;
static std::map<std::array<long, 5>, TuneEntry> g_tune;

// Radix order: 0 = 8s, then 4|2, 3s, 5s; 1 = 4s, then 2, 3s, 5s; 2 = order 0 reversed.
static bool make_sched(int N, int sched, Radices* rd) {
  int n = N, p2 = 0, n3 = 0, n5 = 0, ns = 0;
  while (n % 2 == 0) { n /= 2; ++p2; }
  while (n % 3 == 0) { n /= 3; ++n3; }
  while (n % 5 == 0) { n /= 5; ++n5; }
  if (n != 1) return false;
  int r[32];
  if (sched == 1) {
    for (int i = 0; i < p2 / 2; ++i) r[ns++] = 4;
    if (p2 % 2) r[ns++] = 2;
  } else {
    for (int i = 0; i < p2 / 3; ++i) r[ns++] = 8;
    if (p2 % 3 == 2) r[ns++] = 4;
    if (p2 % 3 == 1) r[ns++] = 2;
  }
  for (int i = 0; i < n3; ++i) r[ns++] = 3;
  for (int i = 0; i < n5; ++i) r[ns++] = 5;
  if (ns > 16) return false;
  rd->n = ns;
  for (int i = 0; i < ns; ++i) rd->r[i] = sched == 2 ? r[ns - 1 - i] : r[i];
  return true;
}

static bool is_capturing(cudaStream_t st) {
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(st, &cs) != cudaSuccess) {
    cudaGetLastError();
    return true;   // unknown: behave as if capturing (no tuning)
  }
  return cs != cudaStreamCaptureStatusNone;
}

// Launch one candidate. Returns FIT_OK, 1 (candidate not available) or an error code.
template <typename T>
static int launch_cand(int kind, const void* in, void* out, const Axis& ax, long P, long Q, T scale, const Cand& c,
                       cudaStream_t st) {
  typedef typename Vec2<T>::t V;
  const V* tw = axis_tw<T>(ax);
  const int N = ax.N;
  if (c.engine == 0) {
    if (kind == PASS_FWD || kind == PASS_INV)
      return ct_strided<T>((const V*)in, (V*)out, N, P, Q, kind == PASS_INV, scale, tw, st);
    if (kind == PASS_C2R) return ct_c2r<T>((const V*)in, (T*)out, N, P, scale, tw, st);
    return ct_r2c<T>((const T*)in, (V*)out, N, P, scale, tw, st);
  }
  Radices rd;
  if (!make_sched(N, c.sched, &rd)) return 1;
  const long E = (long)c.C * N;
  long nthr = (E + c.ept - 1) / c.ept;
  nthr = ((nthr + 31) / 32) * 32;
  if (nthr < 32) nthr = 32;
  const size_t smem = (size_t)(E + N) * sizeof(V);
  if (nthr > 1024 || smem > 200 * 1024) return 1;
  if (kind == PASS_FWD || kind == PASS_INV) {
    const long tpq = (P + c.C - 1) / c.C;
    const long grid = tpq * Q;
    if (grid > 2147483647L) return 1;
#define FIT_TS(INV, EPT)                                                                                      \
  do {                                                                                                        \
    FIT_TRY(prep_kernel(k_pass_strided<V, INV, EPT>, smem, (int)nthr));                                                  \
    k_pass_strided<V, INV, EPT><<<(unsigned)grid, (unsigned)nthr, smem, st>>>((const V*)in, (V*)out, N, P, tpq, \
                                                                               c.C, rd, tw, scale);           \
  } while (0)
    if (kind == PASS_INV) {
      if (c.ept == 8) FIT_TS(true, 8); else FIT_TS(true, 16);
    } else {
      if (c.ept == 8) FIT_TS(false, 8); else FIT_TS(false, 16);
    }
#undef FIT_TS
    return FIT_OK;
  }
  const long grid = (P + 2L * c.C - 1) / (2L * c.C);
  if (kind == PASS_C2R) {
    if (c.ept == 8) {
      FIT_TRY(prep_kernel(k_c2r_x<V, 8>, smem, (int)nthr));
      k_c2r_x<V, 8><<<(unsigned)grid, (unsigned)nthr, smem, st>>>((const V*)in, (T*)out, N, P, c.C, rd, tw, scale);
    } else {
      FIT_TRY(prep_kernel(k_c2r_x<V, 16>, smem, (int)nthr));
      k_c2r_x<V, 16><<<(unsigned)grid, (unsigned)nthr, smem, st>>>((const V*)in, (T*)out, N, P, c.C, rd, tw, scale);
    }
  } else {
    if (c.ept == 8) {
      FIT_TRY(prep_kernel(k_r2c_x<V, 8>, smem, (int)nthr));
      k_r2c_x<V, 8><<<(unsigned)grid, (unsigned)nthr, smem, st>>>((const T*)in, (V*)out, N, P, c.C, rd, tw, scale);
    } else {
      FIT_TRY(prep_kernel(k_r2c_x<V, 16>, smem, (int)nthr));
      k_r2c_x<V, 16><<<(unsigned)grid, (unsigned)nthr, smem, st>>>((const T*)in, (V*)out, N, P, c.C, rd, tw, scale);
    }
  }
  return FIT_OK;
}

// Bytes of the input and output buffers of a pass (P columns or lines, Q batches).
template <typename T>
static void pass_bytes(int kind, int N, long P, long Q, size_t* bin, size_t* bout) {
  typedef typename Vec2<T>::t V;
  if (kind == PASS_FWD || kind == PASS_INV) {
    *bin = *bout = sizeof(V) * (size_t)P * N * Q;
  } else if (kind == PASS_C2R) {
    *bin = sizeof(V) * (size_t)P * (N / 2 + 1);
    *bout = sizeof(T) * (size_t)P * N;
  } else {
    *bin = sizeof(T) * (size_t)P * N;
    *bout = sizeof(V) * (size_t)P * (N / 2 + 1);
  }
}

// The choice for this pass shape: true with *c set when the tuner is on and a choice exists (made
// now if needed and possible); false means "use the default path".
template <typename T>
static bool tune_pick(int kind, const Axis& ax, long P, long Q, T scale, cudaStream_t st, Cand* c) {
  typedef typename Vec2<T>::t V;
  if (!g_tune_on.load()) return false;
  const std::array<long, 5> key = {kind, ax.N, P, Q, (long)sizeof(V)};
  {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    auto it = g_tune.find(key);
    if (it != g_tune.end()) {
      *c = it->second.best;
      return true;
    }
  }
  if (is_capturing(st)) return false;
  // Scratch: the batch dimension Q is cut so a tuning buffer stays under 256 MB (every block
  // handles one (tile, q) pair, so per-q cost is what is compared).
  long Qt = Q;
  size_t bin, bout;
  pass_bytes<T>(kind, ax.N, P, 1, &bin, &bout);
  const size_t cap = 256u << 20;
  if (kind == PASS_FWD || kind == PASS_INV) {
    while (Qt > 1 && bin * Qt > cap) Qt = (Qt + 1) / 2;
  }
  pass_bytes<T>(kind, ax.N, P, Qt, &bin, &bout);
  void *sin = nullptr, *sout = nullptr;
  if (cudaMalloc(&sin, bin) != cudaSuccess || cudaMalloc(&sout, bout) != cudaSuccess) {
    cudaGetLastError();
    if (sin) cudaFree(sin);
    return false;
  }
  cudaMemsetAsync(sin, 0, bin, st);
  std::vector<Cand> cands;
  cands.push_back(Cand{0, 0, 0, 0});
  const int vb = (int)sizeof(V);
  for (int C = 1; C <= 256; C *= 2) {
    if ((long)C * ax.N * vb > 192 * 1024) break;
    for (int ept : {8, 16})
      for (int sched = 0; sched < 3; ++sched) cands.push_back(Cand{1, C, ept, sched});
  }
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  TuneEntry best;
  best.ms_best = 1e30f;
  best.ms_default = -1.f;
  best.ncand = 0;
  best.best = Cand{0, 0, 0, 0};
  bool have = false;
  for (const Cand& cd : cands) {
    if (cd.engine == 1 && cd.C > 1) {
      const long cols = (kind == PASS_FWD || kind == PASS_INV) ? P : (P + 1) / 2;
      long ap2 = 1;
      while (ap2 < cols) ap2 *= 2;
      if (cd.C > ap2) continue;   // wider than the columns (line pairs) that exist
    }
    int rc = launch_cand<T>(kind, sin, sout, ax, P, Qt, scale, cd, st);
    if (rc == 1) continue;
    if (rc != FIT_OK || cudaGetLastError() != cudaSuccess) continue;
    cudaEventRecord(e0, st);
    for (int r = 0; r < 3; ++r) launch_cand<T>(kind, sin, sout, ax, P, Qt, scale, cd, st);
    cudaEventRecord(e1, st);
    if (cudaEventSynchronize(e1) != cudaSuccess || cudaGetLastError() != cudaSuccess) continue;
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    ms /= 3.f;
    best.ncand++;
    if (cd.engine == 0 && best.ms_default < 0.f) best.ms_default = ms;
    if (ms < best.ms_best) {
      best.ms_best = ms;
      best.best = cd;
      have = true;
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(sin);
  cudaFree(sout);
  if (!have) return false;
  if (best.ms_default < 0.f) best.ms_default = best.ms_best;   // no compile-time kernel for this length
  std::lock_guard<std::mutex> lk(g_tune_mu);
  g_tune[key] = best;
  *c = best.best;
  return true;
}

void autotune_enable(bool on) { g_tune_on.store(on ? 1 : 0); }

void autotune_clear() {
  std::lock_guard<std::mutex> lk(g_tune_mu);
  g_tune.clear();
}

// entries, entries whose choice is not the compile-time kernel, sum of default ms, sum of best ms
void autotune_summary(long* n, long* changed, double* ms_default, double* ms_best) {
  std::lock_guard<std::mutex> lk(g_tune_mu);
  *n = (long)g_tune.size();
  *changed = 0;
  *ms_default = *ms_best = 0.0;
  for (auto& kv : g_tune) {
    if (kv.second.best.engine != 0) ++*changed;
    *ms_default += kv.second.ms_default;
    *ms_best += kv.second.ms_best;
  }
}

// Entry i: kind, N, P, Q, element bytes, engine, C, ept, sched; times in ms.
bool autotune_entry(long i, long* fields, float* ms_best, float* ms_default) {
  std::lock_guard<std::mutex> lk(g_tune_mu);
  if (i < 0 || i >= (long)g_tune.size()) return false;
  auto it = g_tune.begin();
  std::advance(it, i);
  for (int k = 0; k < 5; ++k) fields[k] = it->first[k];
  fields[5] = it->second.best.engine;
  fields[6] = it->second.best.C;
  fields[7] = it->second.best.ept;
  fields[8] = it->second.best.sched;
  *ms_best = it->second.ms_best;
  *ms_default = it->second.ms_default;
  return true;
}

template <typename T>
int pass_strided(const typename Vec2<T>::t* in, typename Vec2<T>::t* out, const Axis& ax, long P, long Q,
                 bool inverse, T scale, cudaStream_t st) {
  typedef typename Vec2<T>::t V;
  if (P <= 0 || Q <= 0) return FIT_OK;
  Tile t = pick_tile(ax.N, sizeof(V), P);
  if (t.nthr > 1024) {
    fit_set_error("tile too large");
    return FIT_ERR_SIZE;
  }
  const long tpq = (P + t.C - 1) / t.C;
  const long grid = tpq * Q;
  if (grid > 2147483647L) {
    fit_set_error("grid too large");
    return FIT_ERR_SIZE;
  }
  const V* tw = axis_tw<T>(ax);
  fit_prof_begin(PK_FFT_STRIDED, 2.0 * (double)P * ax.N * Q * sizeof(V), st);
  {
    Cand c;
    if (tune_pick<T>(inverse ? PASS_INV : PASS_FWD, ax, P, Q, scale, st, &c)) {
      const int rc = launch_cand<T>(inverse ? PASS_INV : PASS_FWD, in, out, ax, P, Q, scale, c, st);
      if (rc == FIT_OK) {
        fit_prof_end(st);
        FIT_LAUNCH_CHECK();
        return FIT_OK;
      }
      if (rc != 1) return rc;
    }
  }
  {
    const int rc = ct_strided<T>(in, out, ax.N, P, Q, inverse, scale, tw, st);
    if (rc != 1) {
      fit_prof_end(st);
      if (rc != FIT_OK) return rc;
      FIT_LAUNCH_CHECK();
      return FIT_OK;
    }
  }
#define FIT_PS_LAUNCH(INV, EPT)                                                                          \
  do {                                                                                                 \
    FIT_TRY(prep_kernel(k_pass_strided<V, INV, EPT>, t.smem, t.nthr));                                         \
    k_pass_strided<V, INV, EPT><<<(unsigned)grid, t.nthr, t.smem, st>>>(in, out, ax.N, P, tpq, t.C, ax.rd, tw, \
                                                                          scale);                      \
  } while (0)
  if (inverse) {
    if (t.EPT == 8) FIT_PS_LAUNCH(true, 8); else FIT_PS_LAUNCH(true, 16);
  } else {
    if (t.EPT == 8) FIT_PS_LAUNCH(false, 8); else FIT_PS_LAUNCH(false, 16);
  }
#undef FIT_PS_LAUNCH
  fit_prof_end(st);
  FIT_LAUNCH_CHECK();
  return FIT_OK;
}

template <typename T>
int pass_c2r_x(const typename Vec2<T>::t* in, T* out, const Axis& ax, long L, T scale, cudaStream_t st) {
  typedef typename Vec2<T>::t V;
  if (L <= 0) return FIT_OK;
  Tile t = pick_tile(ax.N, sizeof(V), (L + 1) / 2);
  const long grid = (L + 2L * t.C - 1) / (2L * t.C);
  const V* tw = axis_tw<T>(ax);
  fit_prof_begin(PK_FFT_C2R_X, (double)L * ((ax.N / 2 + 1) * sizeof(V) + ax.N * sizeof(T)), st);
  {
    Cand c;
    if (tune_pick<T>(PASS_C2R, ax, L, 1, scale, st, &c)) {
      const int rc = launch_cand<T>(PASS_C2R, in, out, ax, L, 1, scale, c, st);
      if (rc == FIT_OK) {
        fit_prof_end(st);
        FIT_LAUNCH_CHECK();
        return FIT_OK;
      }
      if (rc != 1) return rc;
    }
  }
  {
    const int rc = ct_c2r<T>(in, out, ax.N, L, scale, tw, st);
    if (rc != 1) {
      fit_prof_end(st);
      if (rc != FIT_OK) return rc;
      FIT_LAUNCH_CHECK();
      return FIT_OK;
    }
  }
  if (t.EPT == 8) {
    FIT_TRY(prep_kernel(k_c2r_x<V, 8>, t.smem, t.nthr));
    k_c2r_x<V, 8><<<(unsigned)grid, t.nthr, t.smem, st>>>(in, out, ax.N, L, t.C, ax.rd, tw, scale);
  } else {
    FIT_TRY(prep_kernel(k_c2r_x<V, 16>, t.smem, t.nthr));
    k_c2r_x<V, 16><<<(unsigned)grid, t.nthr, t.smem, st>>>(in, out, ax.N, L, t.C, ax.rd, tw, scale);
  }
  fit_prof_end(st);
  FIT_LAUNCH_CHECK();
  return FIT_OK;
}

template <typename T>
int pass_r2c_x(const T* in, typename Vec2<T>::t* out, const Axis& ax, long L, T scale, cudaStream_t st) {
  typedef typename Vec2<T>::t V;
  if (L <= 0) return FIT_OK;
  Tile t = pick_tile(ax.N, sizeof(V), (L + 1) / 2);
  const long grid = (L + 2L * t.C - 1) / (2L * t.C);
  const V* tw = axis_tw<T>(ax);
  fit_prof_begin(PK_FFT_R2C_X, (double)L * ((ax.N / 2 + 1) * sizeof(V) + ax.N * sizeof(T)), st);
  {
    Cand c;
    if (tune_pick<T>(PASS_R2C, ax, L, 1, scale, st, &c)) {
      const int rc = launch_cand<T>(PASS_R2C, in, out, ax, L, 1, scale, c, st);
      if (rc == FIT_OK) {
        fit_prof_end(st);
        FIT_LAUNCH_CHECK();
        return FIT_OK;
      }
      if (rc != 1) return rc;
    }
  }
  {
    const int rc = ct_r2c<T>(in, out, ax.N, L, scale, tw, st);
    if (rc != 1) {
      fit_prof_end(st);
      if (rc != FIT_OK) return rc;
      FIT_LAUNCH_CHECK();
      return FIT_OK;
    }
  }
  if (t.EPT == 8) {
    FIT_TRY(prep_kernel(k_r2c_x<V, 8>, t.smem, t.nthr));
    k_r2c_x<V, 8><<<(unsigned)grid, t.nthr, t.smem, st>>>(in, out, ax.N, L, t.C, ax.rd, tw, scale);
  } else {
    FIT_TRY(prep_kernel(k_r2c_x<V, 16>, t.smem, t.nthr));
    k_r2c_x<V, 16><<<(unsigned)grid, t.nthr, t.smem, st>>>(in, out, ax.N, L, t.C, ax.rd, tw, scale);
  }
  fit_prof_end(st);
  FIT_LAUNCH_CHECK();
  return FIT_OK;
}

// half (nf fields, destroyed) -> phys (nf fields); x is the last (real) pass.
template <typename T>
int inverse_nd(typename Vec2<T>::t* half, T* phys, const GridDesc& g, const Axis* ax, long nf, T scale,
               cudaStream_t st) {
  const long Mh0 = g.Mh0, M1 = g.M[1], M2 = g.M[2];
  if (g.nd == 3) FIT_TRY(pass_strided<T>(half, half, ax[2], Mh0 * M1, nf, true, (T)1, st));
  if (g.nd >= 2) FIT_TRY(pass_strided<T>(half, half, ax[1], Mh0, M2 * nf, true, (T)1, st));
  FIT_TRY(pass_c2r_x<T>(half, phys, ax[0], M1 * M2 * nf, scale, st));
  return FIT_OK;
}

template <typename T>
int forward_nd(const T* phys, typename Vec2<T>::t* half, const GridDesc& g, const Axis* ax, long nf, T scale,
               cudaStream_t st) {
  const long Mh0 = g.Mh0, M1 = g.M[1], M2 = g.M[2];
  FIT_TRY(pass_r2c_x<T>(phys, half, ax[0], M1 * M2 * nf, scale, st));
  if (g.nd >= 2) FIT_TRY(pass_strided<T>(half, half, ax[1], Mh0, M2 * nf, false, (T)1, st));
  if (g.nd == 3) FIT_TRY(pass_strided<T>(half, half, ax[2], Mh0 * M1, nf, false, (T)1, st));
  return FIT_OK;
}

template <typename T>
int forward_nd_full(const T* phys, typename Vec2<T>::t* half, typename Vec2<T>::t* full, const GridDesc& g,
                    const Axis* ax, long nf, T scale, cudaStream_t st) {
  if (g.nd != 3 || g.padded) return 1;
  const int n2 = g.M[2];
  bool ct = false;
  for (int n : {8, 12, 16, 24, 32, 48, 64, 96, 128, 192, 256, 384, 512, 768, 1024}) ct = ct || n == n2;
  if (!ct) return 1;
  const long Mh0 = g.Mh0, M1 = g.M[1], M2 = g.M[2];
  FIT_TRY(pass_r2c_x<T>(phys, half, ax[0], M1 * M2 * nf, scale, st));
  FIT_TRY(pass_strided<T>(half, half, ax[1], Mh0, M2 * nf, false, (T)1, st));
  fit_prof_begin(PK_FFT_Z_FULL, (double)nf * Mh0 * M1 * M2 * sizeof(typename Vec2<T>::t) * 3.0, st);
  const int rc = ct_z_full<T>(half, full, g.M[0], (int)Mh0, (int)M1, n2, nf, axis_tw<T>(ax[2]), st);
  fit_prof_end(st);
  if (rc != FIT_OK) return rc == 1 ? FIT_ERR_SIZE : rc;
  FIT_LAUNCH_CHECK();
  return FIT_OK;
}

template int forward_nd_full<float>(const float*, float2*, float2*, const GridDesc&, const Axis*, long, float,
                                    cudaStream_t);
template int forward_nd_full<double>(const double*, double2*, double2*, const GridDesc&, const Axis*, long, double,
                                     cudaStream_t);
template int pass_strided<float>(const float2*, float2*, const Axis&, long, long, bool, float, cudaStream_t);
template int pass_strided<double>(const double2*, double2*, const Axis&, long, long, bool, double, cudaStream_t);
template int pass_c2r_x<float>(const float2*, float*, const Axis&, long, float, cudaStream_t);
template int pass_c2r_x<double>(const double2*, double*, const Axis&, long, double, cudaStream_t);
template int pass_r2c_x<float>(const float*, float2*, const Axis&, long, float, cudaStream_t);
template int pass_r2c_x<double>(const double*, double2*, const Axis&, long, double, cudaStream_t);
template int inverse_nd<float>(float2*, float*, const GridDesc&, const Axis*, long, float, cudaStream_t);
template int inverse_nd<double>(double2*, double*, const GridDesc&, const Axis*, long, double, cudaStream_t);
template int forward_nd<float>(const float*, float2*, const GridDesc&, const Axis*, long, float, cudaStream_t);
template int forward_nd<double>(const double*, double2*, const GridDesc&, const Axis*, long, double, cudaStream_t);

}  // namespace fit
