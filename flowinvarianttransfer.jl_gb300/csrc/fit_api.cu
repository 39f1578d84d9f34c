// C ABI of libfit_gb300 (declared in include/fit_gb300.h): plan lifetime, the generic
// nonlinear-term pipeline, and the diagnostic entry points built on it.
#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <string.h>

#include <atomic>
#include <mutex>
#include <thread>
#include <vector>

#include "fit_gb300.h"
#include "fit_plan.cuh"

// ---- errors and launch accounting -------------------------------------------------------------

static thread_local char g_err[1024] = "";
static std::atomic<long long> g_launches(0);

// ---- per-launch profiling ------------------------------------------------------------------------
struct ProfRec {
  int kind;
  double bytes;
  cudaEvent_t a, b;
};
static std::mutex g_prof_mu;
static std::vector<ProfRec> g_prof;
static std::vector<cudaEvent_t> g_prof_pool;
static size_t g_prof_used = 0;
static bool g_prof_enabled = false;
static const char* g_prof_names[PK_COUNT] = {"fft_strided", "fft_c2r_x", "fft_r2c_x", "gather", "product",
                                             "bin", "carrier", "triad", "shell_table", "s2s_zinv", "s2s_yinv",
                                             "s2s_xmix", "s2s_yfwd", "s2s_zfwd_bin", "s2s_velocity",
                                             "fft_z_full"};

static cudaEvent_t prof_event() {
  if (g_prof_used < g_prof_pool.size()) return g_prof_pool[g_prof_used++];
  cudaEvent_t e;
  if (cudaEventCreate(&e) != cudaSuccess) return nullptr;
  g_prof_pool.push_back(e);
  ++g_prof_used;
  return e;
}

bool fit_prof_on() { return g_prof_enabled; }

void fit_prof_begin(int kind, double bytes, cudaStream_t st) {
  if (!g_prof_enabled) return;
  std::lock_guard<std::mutex> lk(g_prof_mu);
  ProfRec r;
  r.kind = kind;
  r.bytes = bytes;
  r.a = prof_event();
  r.b = prof_event();
  if (!r.a || !r.b) return;
  cudaEventRecord(r.a, st);
  g_prof.push_back(r);
}

void fit_prof_end(cudaStream_t st) {
  if (!g_prof_enabled) return;
  std::lock_guard<std::mutex> lk(g_prof_mu);
  if (!g_prof.empty()) cudaEventRecord(g_prof.back().b, st);
}

void fit_set_error(const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof(g_err), fmt, ap);
  va_end(ap);
}
const char* fit_get_error() { return g_err; }
void fit_count_launches(long n) { g_launches += n; }
long fit_launch_total() { return (long)g_launches.load(); }

long long fit_wait_cycles() {
  const char* v = getenv("FIT_TEST_WAIT_CYCLES");
  if (v && v[0]) {
    const long long c = atoll(v);
    if (c > 0) return c;
  }
  return FIT_WAIT_CYCLES;
}

#define API_CHECK(cond, code, ...)  \
  do {                              \
    if (!(cond)) {                  \
      fit_set_error(__VA_ARGS__);   \
      return code;                  \
    }                               \
  } while (0)

namespace fit {

int ensure(fit_plan* p, fit_dbuf* b, size_t bytes) {
  if (bytes == 0) bytes = 16;
  if (b->cap >= bytes) return FIT_OK;
  if (b->p) {
    cudaFree(b->p);
    p->bytes -= b->cap;
    b->p = nullptr;
    b->cap = 0;
  }
  cudaError_t e = cudaMalloc(&b->p, bytes);
  if (e != cudaSuccess) {
    b->p = nullptr;
    fit_set_error("cudaMalloc(%zu bytes) failed: %s", bytes, cudaGetErrorString(e));
    return FIT_ERR_ALLOC;
  }
  b->cap = bytes;
  p->bytes += bytes;
  p->buf_gen++;
  return FIT_OK;
}

static void release(fit_dbuf* b) {
  if (b->p) cudaFree(b->p);
  b->p = nullptr;
  b->cap = 0;
}

int ensure_shells(fit_plan* p, const double* edges, int n_edges, unsigned dims, int coord_f32) {
  API_CHECK(n_edges >= 1, FIT_ERR_ARG, "need at least one shell edge");
  API_CHECK(edges != nullptr, FIT_ERR_ARG, "edges is NULL");
  for (int i = 1; i < n_edges; ++i)
    API_CHECK(edges[i] >= edges[i - 1], FIT_ERR_ARG, "shell edges must be monotonically increasing");
  const unsigned all = (1u << p->nd) - 1u;
  if (dims == 0) dims = all;
  API_CHECK((dims & ~all) == 0, FIT_ERR_ARG, "ShellMagnitude dims mask 0x%x out of range for nd=%d spatial dimensions.",
            dims, p->nd);
  bool same = p->cached_f32 == coord_f32 && p->cached_dims == dims && (int)p->cached_edges.size() == n_edges &&
              memcmp(p->cached_edges.data(), edges, sizeof(double) * n_edges) == 0;
  if (same) return FIT_OK;
  FIT_TRY(ensure(p, &p->shell_full, sizeof(uint16_t) * p->g.Ntot));
  FIT_TRY(ensure(p, &p->edges_dev, sizeof(double) * n_edges));
  FIT_CUDA_CHECK(cudaMemcpyAsync(p->edges_dev.p, edges, sizeof(double) * n_edges, cudaMemcpyHostToDevice, p->stream));
  FIT_TRY(shell_table(p->g, p->kt, dims, (const double*)p->edges_dev.p, n_edges, coord_f32,
                      (uint16_t*)p->shell_full.p, p->stream));
  p->cached_edges.assign(edges, edges + n_edges);
  p->cached_dims = dims;
  p->cached_f32 = coord_f32;
  p->nsh = n_edges - 1;
  p->shell_gen++;
  std::vector<uint16_t>().swap(p->idx_host);
  return FIT_OK;
}

// N̂ half spectrum (M fields) into p->nh. band > 0 restricts the advected field to that shell
// (the shell-to-shell mediator); reuse_u keeps the advecting velocity from the previous call.
template <typename T>
int nonlinear_half(fit_plan* p, const void* f_dev, const void* a_dev, int band, bool reuse_u, int wband) {
  typedef typename Vec2<T>::t V;
  const GridDesc& g = p->g;
  const int nd = p->nd, M = p->M;
  const long nfu = nd, nfg = (long)M * nd;
  FIT_TRY(ensure(p, &p->hs, sizeof(V) * (nfu + nfg) * g.Mhalf));
  FIT_TRY(ensure(p, &p->ph, sizeof(T) * (nfu + nfg) * g.Mtot));
  FIT_TRY(ensure(p, &p->nph, sizeof(T) * M * g.Mtot));
  FIT_TRY(ensure(p, &p->nh, sizeof(V) * M * g.Mhalf));
  V* hs = (V*)p->hs.p;
  T* ph = (T*)p->ph.p;
  GatherArgs a;
  memset(&a, 0, sizeof(a));
  a.src[0] = f_dev;
  a.src[1] = a_dev;
  a.src_comp_stride[0] = g.Ntot;
  a.src_comp_stride[1] = g.Ntot;
  a.in_f64 = p->io_f64;
  a.two_thirds = p->dealias == 1;
  a.shell_full = (const uint16_t*)p->shell_full.p;
  a.scale = 1.0;
  const T inv_m = (T)(1.0 / (double)g.Mtot);
  if (!reuse_u) {
    a.nfields = nd;
    for (int j = 0; j < nd; ++j) a.f[j] = GatherField{1, j, -1, 0};
    FIT_TRY(gather_half<T>(g, p->kt, a, hs, p->stream));
    FIT_TRY(inverse_nd<T>(hs, ph, g, p->ax, nfu, inv_m, p->stream));
  }
  a.nfields = (int)nfg;
  a.wtab = p->wtab.p;
  a.w_f64 = p->prec == 64;
  for (int c = 0; c < M; ++c)
    for (int j = 0; j < nd; ++j) a.f[c * nd + j] = GatherField{0, c, j, band, 0, wband};
  FIT_TRY(gather_half<T>(g, p->kt, a, hs + nfu * g.Mhalf, p->stream));
  FIT_TRY(inverse_nd<T>(hs + nfu * g.Mhalf, ph + nfu * g.Mtot, g, p->ax, nfg, inv_m, p->stream));
  FIT_TRY(product<T>(ph, ph + nfu * g.Mtot, (T*)p->nph.p, nd, M, g.Mtot, p->stream));
  const double fs = g.padded ? (double)g.Mtot / ((double)g.Ntot * (double)g.Ntot) : 1.0 / (double)g.Ntot;
  FIT_TRY(forward_nd<T>((const T*)p->nph.p, (V*)p->nh.p, g, p->ax, M, (T)fs, p->stream));
  return FIT_OK;
}

template int nonlinear_half<float>(fit_plan*, const void*, const void*, int, bool, int);
template int nonlinear_half<double>(fit_plan*, const void*, const void*, int, bool, int);

}  // namespace fit

using namespace fit;

// ---- helpers ------------------------------------------------------------------------------------

static size_t cbytes(const fit_plan* p) { return p->io_f64 ? 16 : 8; }

// Device view of a user array: the pointer itself (device) or a staged copy (host).
static int stage_in(fit_plan* p, fit_dbuf* b, const void* src, size_t bytes, int ptr_kind, const void** out) {
  if (src == nullptr) {
    *out = nullptr;
    return FIT_OK;
  }
  if (ptr_kind == FIT_PTR_DEVICE) {
    *out = src;
    return FIT_OK;
  }
  FIT_TRY(ensure(p, b, bytes));
  FIT_CUDA_CHECK(cudaMemcpyAsync(b->p, src, bytes, cudaMemcpyHostToDevice, p->stream));
  p->h2d_total += bytes;
  *out = b->p;
  return FIT_OK;
}

// Host inputs of a path that reads only the 2/3-kept modes: copy just the box of modes every axis
// keeps (indices [0, K] and [N - K, N) per axis). Pinned host memory the device can address is read
// by a kernel over the host link (one launch over the box's row runs; steadier and faster than the
// copy engines on a coherent host link); other host memory goes through 8 pitched 3D copies per
// component (one per octant of the box). Modes outside the box are left unwritten in the staging
// buffer and are never read. FIT_KEPT_BOX_COPY_ENGINE=1 selects the 3D copies for pinned memory too.
// With `defer`, a pinned field is not read here: the shell-to-shell step reads it into the staging
// buffer itself (p->kept_src), overlapping the read with its first passes.
static int stage_in_kept_box(fit_plan* p, fit_dbuf* b, const void* src, size_t bytes, int ncomp, const void** out,
                             bool defer = false) {
  if (src == nullptr) {
    *out = nullptr;
    return FIT_OK;
  }
  FIT_TRY(ensure(p, b, bytes));
  const GridDesc& g = p->g;
  const size_t eb = cbytes(p), row = eb * g.N[0], plane = row * g.N[1];
  cudaPointerAttributes at;
  const char* env = getenv("FIT_KEPT_BOX_COPY_ENGINE");
  const bool dma = env && env[0] == '1';
  if (!dma && cudaPointerGetAttributes(&at, src) == cudaSuccess && at.type == cudaMemoryTypeHost &&
      at.devicePointer != nullptr && ((uintptr_t)at.devicePointer % eb) == 0) {
    if (defer) p->kept_src = at.devicePointer;
    else FIT_TRY(copy_kept_box(at.devicePointer, b->p, g.N, ncomp, (int)eb, p->stream));
    long kept = 1;
    for (int d = 0; d < 3; ++d) kept *= 2L * (g.N[d] / 3 - 1) + 1;
    p->h2d_total += (size_t)kept * ncomp * eb;
    *out = b->p;
    return FIT_OK;
  }
  cudaGetLastError();   // an unregistered pointer leaves an error from the attribute query
  int lo[3][2], n[3][2];
  for (int d = 0; d < 3; ++d) {
    const int K = g.N[d] / 3 - 1;   // kept iff min(k, N - k) < N / 3
    lo[d][0] = 0;
    n[d][0] = K + 1;
    lo[d][1] = g.N[d] - K;
    n[d][1] = K;
  }
  for (int c = 0; c < ncomp; ++c) {
    char* dst = (char*)b->p + (size_t)c * plane * g.N[2];
    const char* hs = (const char*)src + (size_t)c * plane * g.N[2];
    for (int o = 0; o < 8; ++o) {
      const int rx = o & 1, ry = (o >> 1) & 1, rz = o >> 2;
      if (n[0][rx] <= 0 || n[1][ry] <= 0 || n[2][rz] <= 0) continue;
      cudaMemcpy3DParms cp;
      memset(&cp, 0, sizeof(cp));
      cp.srcPtr = make_cudaPitchedPtr((void*)hs, row, row, g.N[1]);
      cp.dstPtr = make_cudaPitchedPtr(dst, row, row, g.N[1]);
      cp.srcPos = make_cudaPos((size_t)lo[0][rx] * eb, lo[1][ry], lo[2][rz]);
      cp.dstPos = cp.srcPos;
      cp.extent = make_cudaExtent((size_t)n[0][rx] * eb, n[1][ry], n[2][rz]);
      cp.kind = cudaMemcpyHostToDevice;
      FIT_CUDA_CHECK(cudaMemcpy3DAsync(&cp, p->stream));
      p->h2d_total += (size_t)n[0][rx] * eb * n[1][ry] * n[2][rz];
    }
  }
  *out = b->p;
  return FIT_OK;
}

static int copy_out(fit_plan* p, void* dst, const void* dev, size_t bytes, int ptr_kind) {
  if (dst == nullptr) return FIT_OK;
  FIT_CUDA_CHECK(cudaMemcpyAsync(dst, dev, bytes, ptr_kind == FIT_PTR_DEVICE ? cudaMemcpyDeviceToDevice
                                                                             : cudaMemcpyDeviceToHost,
                                 p->stream));
  return FIT_OK;
}

static int sync_plan(fit_plan* p) {
  FIT_CUDA_CHECK(cudaStreamSynchronize(p->stream));
  FIT_CUDA_CHECK(cudaGetLastError());
  return FIT_OK;
}

static int check_invariant(const fit_plan* p, int inv, int ncomp) {
  API_CHECK(inv >= 0 && inv <= 3, FIT_ERR_ARG, "unknown invariant %d", inv);
  if (inv == INV_HELICITY)
    API_CHECK(p->nd == 3 && ncomp == 3, FIT_ERR_ARG, "Helicity transfer is defined in 3D only (got nd=%d).", p->nd);
  if (inv == INV_ENSTROPHY)
    API_CHECK((p->nd == 2 || p->nd == 3) && ncomp == p->nd, FIT_ERR_ARG,
              "Enstrophy transfer is defined in 2D (scalar vorticity, conserved) or 3D (vector vorticity); got nd=%d.",
              p->nd);
  return FIT_OK;
}

template <typename T>
int fit::carrier_and_bin_setup(fit_plan* p, const void* carrier, int inv) {
  typedef typename Vec2<T>::t V;
  FIT_TRY(ensure(p, &p->ceff, sizeof(V) * 3 * p->g.Mhalf));
  FIT_TRY(ensure(p, &p->seff, sizeof(uint16_t) * p->g.Mhalf));
  return effective_carrier<T>(p->g, p->kt, carrier, p->io_f64, p->g.Ntot, p->M, inv, p->dealias == 1,
                              (const uint16_t*)p->shell_full.p, (V*)p->ceff.p, p->M, (uint16_t*)p->seff.p,
                              p->stream);
}

template <typename T>
int fit::bin_into(fit_plan* p, const void* nh, long bstride, int nb, const void* ceff, double* out) {
  typedef typename Vec2<T>::t V;
  const long cap = 2L * 152 * nb * p->nsh;
  FIT_TRY(ensure(p, &p->partial, sizeof(double) * cap));
  return bin_density<T>(p->g, (const V*)nh, bstride, nb, (const V*)ceff, p->M, (const uint16_t*)p->seff.p, p->nsh,
                        (double*)p->partial.p, cap, out, p->stream);
}

template int fit::carrier_and_bin_setup<float>(fit_plan*, const void*, int);
template int fit::carrier_and_bin_setup<double>(fit_plan*, const void*, int);
template int fit::bin_into<float>(fit_plan*, const void*, long, int, const void*, double*);
template int fit::bin_into<double>(fit_plan*, const void*, long, int, const void*, double*);

// ---- C ABI ------------------------------------------------------------------------------------

extern "C" {

const char* fit_last_error(void) { return fit_get_error(); }

int fit_prof_enable(int on) {
  std::lock_guard<std::mutex> lk(g_prof_mu);
  cudaDeviceSynchronize();
  g_prof.clear();
  g_prof_used = 0;
  g_prof_enabled = on != 0;
  return FIT_OK;
}

const char* fit_prof_kind_name(int kind) { return (kind >= 0 && kind < PK_COUNT) ? g_prof_names[kind] : ""; }

int fit_prof_read(int kind, double* ms_total, double* bytes_total, long long* launches) {
  std::lock_guard<std::mutex> lk(g_prof_mu);
  FIT_CUDA_CHECK(cudaDeviceSynchronize());
  double ms = 0.0, by = 0.0;
  long long n = 0;
  for (const ProfRec& r : g_prof) {
    if (r.kind != kind) continue;
    float t = 0.f;
    if (cudaEventElapsedTime(&t, r.a, r.b) != cudaSuccess) continue;
    ms += t;
    by += r.bytes;
    ++n;
  }
  if (ms_total) *ms_total = ms;
  if (bytes_total) *bytes_total = by;
  if (launches) *launches = n;
  return FIT_OK;
}
long long fit_launch_count(void) { return g_launches.load(); }

int fit_plan_create(fit_plan** out, int nd, const int64_t* ns, int n_advected, int n_advecting, int dealias,
                    int precision, int io_f64, const double* const* ks) {
  API_CHECK(out != nullptr, FIT_ERR_ARG, "out is NULL");
  *out = nullptr;
  API_CHECK(nd >= 1 && nd <= 3, FIT_ERR_ARG, "nd must be 1, 2 or 3 (got %d)", nd);
  API_CHECK(ns != nullptr && ks != nullptr, FIT_ERR_ARG, "ns/ks is NULL");
  API_CHECK(n_advected >= 1 && n_advected <= 3, FIT_ERR_ARG, "advected field must have 1..3 components");
  API_CHECK(n_advecting >= nd, FIT_ERR_ARG, "advecting velocity needs >= nd components (got %d)", n_advecting);
  API_CHECK(dealias >= 0 && dealias <= 2, FIT_ERR_ARG, "unknown dealiasing %d", dealias);
  API_CHECK(precision == 32 || precision == 64, FIT_ERR_ARG, "precision must be 32 or 64");
  fit_plan* p = new fit_plan();
  p->nd = nd;
  p->M = n_advected;
  p->Dadv = n_advecting;
  p->dealias = dealias;
  p->prec = precision;
  p->io_f64 = io_f64 ? 1 : 0;
  GridDesc& g = p->g;
  g.nd = nd;
  g.padded = dealias == 2;
  for (int d = 0; d < 3; ++d) {
    g.N[d] = d < nd ? (int)ns[d] : 1;
    if (d < nd && ns[d] < 1) {
      delete p;
      fit_set_error("grid size must be positive");
      return FIT_ERR_ARG;
    }
    int m = g.N[d];
    if (g.padded && d < nd) {
      m = (3 * g.N[d] + 1) / 2;
      if ((m - g.N[d]) % 2 != 0) m += 1;   // ext/FlowInvariantTransferFFTWExt.jl:128-131
    }
    g.M[d] = m;
  }
  g.Mh0 = g.M[0] / 2 + 1;
  g.Ntot = (long)g.N[0] * g.N[1] * g.N[2];
  g.Mtot = (long)g.M[0] * g.M[1] * g.M[2];
  g.Mhalf = (long)g.Mh0 * g.M[1] * g.M[2];
  // wavenumbers: must be FFTW order (k[N-i] = -k[i] except at the Nyquist index)
  for (int d = 0; d < nd; ++d) {
    const int N = g.N[d];
    p->ks_host[d].assign(ks[d], ks[d] + N);
    for (int i = 1; i < N; ++i) {
      if (2 * i == N) continue;
      if (!(p->ks_host[d][N - i] == -p->ks_host[d][i])) {
        delete p;
        fit_set_error("ks[%d] is not an FFTW-order wavenumber vector (k[N-i] != -k[i] at i=%d)", d, i);
        return FIT_ERR_ARG;
      }
    }
  }
  int rc = FIT_OK;
  if (cudaStreamCreateWithFlags(&p->stream, cudaStreamNonBlocking) != cudaSuccess) {
    fit_set_error("cudaStreamCreate failed");
    delete p;
    return FIT_ERR_CUDA;
  }
  p->own_stream = true;
  for (int d = 0; d < 3 && rc == FIT_OK; ++d) {
    rc = axis_init(&p->ax[d], g.M[d]);
    p->ax_init[d] = 1;
  }
  for (int d = 0; d < 3 && rc == FIT_OK; ++d) {
    const int N = g.N[d];
    if (cudaMalloc(&p->ks_dev[d], sizeof(double) * N) != cudaSuccess) {
      fit_set_error("cudaMalloc(ks) failed");
      rc = FIT_ERR_ALLOC;
      break;
    }
    std::vector<double> kk(N, 0.0);
    if (d < nd) kk = p->ks_host[d];
    if (cudaMemcpy(p->ks_dev[d], kk.data(), sizeof(double) * N, cudaMemcpyHostToDevice) != cudaSuccess) {
      fit_set_error("ks upload failed");
      rc = FIT_ERR_CUDA;
    }
    p->kt.k[d] = p->ks_dev[d];
    std::vector<float> k32(N);
    for (int i = 0; i < N; ++i) k32[i] = (float)kk[i];
    if (rc == FIT_OK && (cudaMalloc(&p->ks32_dev[d], sizeof(float) * N) != cudaSuccess ||
                         cudaMemcpy(p->ks32_dev[d], k32.data(), sizeof(float) * N, cudaMemcpyHostToDevice) !=
                             cudaSuccess)) {
      fit_set_error("ks upload failed");
      rc = FIT_ERR_CUDA;
    }
    p->kt.k32[d] = p->ks32_dev[d];
  }
  if (rc != FIT_OK) {
    fit_plan_destroy(p);
    return rc;
  }
  *out = p;
  return FIT_OK;
}

int fit_plan_destroy(fit_plan* p) {
  if (!p) return FIT_OK;
  if (p->stream) cudaStreamSynchronize(p->stream);
  s2s_free(p);
  partial_free(p);
  fit_dbuf* bufs[] = {&p->in_u, &p->in_a, &p->in_c, &p->out_c, &p->out_c2, &p->hs, &p->ph, &p->nph, &p->nh,
                      &p->ceff, &p->seff, &p->partial, &p->outd, &p->shell_full, &p->edges_dev, &p->wtab,
                      &p->flag};
  for (fit_dbuf* b : bufs) release(b);
  for (int d = 0; d < 3; ++d) {
    if (p->ax_init[d]) axis_free(&p->ax[d]);
    if (p->ks_dev[d]) cudaFree(p->ks_dev[d]);
    if (p->ks32_dev[d]) cudaFree(p->ks32_dev[d]);
  }
  if (p->own_stream && p->stream) cudaStreamDestroy(p->stream);
  delete p;
  return FIT_OK;
}

int fit_plan_set_stream(fit_plan* p, void* stream) {
  API_CHECK(p != nullptr, FIT_ERR_ARG, "plan is NULL");
  cudaStreamSynchronize(p->stream);
  if (p->own_stream && p->stream) cudaStreamDestroy(p->stream);
  p->own_stream = false;
  p->stream = (cudaStream_t)stream;
  s2s_free(p);   // captured graphs belong to the old stream
  partial_free(p);
  return FIT_OK;
}

int fit_plan_info(const fit_plan* p, int64_t* info, int n) {
  API_CHECK(p != nullptr && info != nullptr, FIT_ERR_ARG, "NULL argument");
  const int64_t v[9] = {p->nd,      p->g.N[0], p->g.N[1], p->g.N[2], p->g.M[0], p->g.M[1], p->g.M[2], (int64_t)p->bytes,
                        (int64_t)p->h2d_total};
  for (int i = 0; i < n && i < 9; ++i) info[i] = v[i];
  return FIT_OK;
}

int fit_nonlinear_term(fit_plan* p, const void* f_hat, const void* adv_hat, void* N_hat, int ptr_kind) {
  API_CHECK(p != nullptr && f_hat != nullptr && N_hat != nullptr, FIT_ERR_ARG, "NULL argument");
  const size_t fb = cbytes(p) * p->g.Ntot * p->M, ab = cbytes(p) * p->g.Ntot * p->Dadv;
  const void *fd, *ad;
  FIT_TRY(stage_in(p, &p->in_u, f_hat, fb, ptr_kind, &fd));
  FIT_TRY(stage_in(p, &p->in_a, adv_hat, ab, ptr_kind, &ad));
  if (!ad) {
    API_CHECK(p->M >= p->nd, FIT_ERR_ARG, "self-advection needs >= nd components");
    ad = fd;
  }
  if (p->prec == 64) FIT_TRY(nonlinear_half<double>(p, fd, ad, 0, false));
  else FIT_TRY(nonlinear_half<float>(p, fd, ad, 0, false));
  void* dst = N_hat;
  if (ptr_kind != FIT_PTR_DEVICE) {
    FIT_TRY(ensure(p, &p->out_c, fb));
    dst = p->out_c.p;
  }
  if (p->prec == 64) FIT_TRY(scatter_full<double>(p->g, (const double2*)p->nh.p, p->M, p->dealias == 1, dst, p->io_f64, p->stream));
  else FIT_TRY(scatter_full<float>(p->g, (const float2*)p->nh.p, p->M, p->dealias == 1, dst, p->io_f64, p->stream));
  if (ptr_kind != FIT_PTR_DEVICE) FIT_TRY(copy_out(p, N_hat, dst, fb, ptr_kind));
  return sync_plan(p);
}

int fit_assign_shells(fit_plan* p, const double* edges, int n_edges, uint32_t dims_mask, int coord_f32,
                      int64_t* idx_out, int ptr_kind) {
  API_CHECK(p != nullptr && idx_out != nullptr, FIT_ERR_ARG, "NULL argument");
  FIT_TRY(ensure_shells(p, edges, n_edges, dims_mask, coord_f32));
  const size_t ob = sizeof(int64_t) * p->g.Ntot;
  int64_t* dst = idx_out;
  if (ptr_kind != FIT_PTR_DEVICE) {
    FIT_TRY(ensure(p, &p->outd, ob));
    dst = (int64_t*)p->outd.p;
  }
  FIT_TRY(shell_table_i64(p->g, (const uint16_t*)p->shell_full.p, dst, p->stream));
  if (ptr_kind != FIT_PTR_DEVICE) FIT_TRY(copy_out(p, idx_out, dst, ob, ptr_kind));
  return sync_plan(p);
}

int fit_transfer_density(fit_plan* p, int invariant, const void* carrier, const void* N_hat, double* t_out,
                         int ptr_kind) {
  API_CHECK(p != nullptr && carrier != nullptr && N_hat != nullptr && t_out != nullptr, FIT_ERR_ARG,
            "NULL argument");
  FIT_TRY(check_invariant(p, invariant, p->M));
  const size_t fb = cbytes(p) * p->g.Ntot * p->M;
  const void *cd, *nd_;
  FIT_TRY(stage_in(p, &p->in_u, carrier, fb, ptr_kind, &cd));
  FIT_TRY(stage_in(p, &p->in_a, N_hat, fb, ptr_kind, &nd_));
  double* dst = t_out;
  const size_t ob = sizeof(double) * p->g.Ntot;
  if (ptr_kind != FIT_PTR_DEVICE) {
    FIT_TRY(ensure(p, &p->outd, ob));
    dst = (double*)p->outd.p;
  }
  FIT_TRY(density_full(p->g, p->kt, cd, nd_, p->io_f64, p->M, invariant, dst, p->stream));
  if (ptr_kind != FIT_PTR_DEVICE) FIT_TRY(copy_out(p, t_out, dst, ob, ptr_kind));
  return sync_plan(p);
}

int fit_spectral_flux(fit_plan* p, const void* u_hat, const void* adv_hat, const void* carrier, const double* edges,
                      int n_edges, uint32_t dims_mask, int coord_f32, int invariant, double* T, double* Pi,
                      int ptr_kind) {
  API_CHECK(p != nullptr && u_hat != nullptr && T != nullptr, FIT_ERR_ARG, "NULL argument");
  FIT_TRY(check_invariant(p, invariant, p->M));
  const size_t fb = cbytes(p) * p->g.Ntot * p->M, ab = cbytes(p) * p->g.Ntot * p->Dadv;
  const void *ud, *ad, *cd;
  FIT_TRY(stage_in(p, &p->in_u, u_hat, fb, ptr_kind, &ud));
  FIT_TRY(stage_in(p, &p->in_a, adv_hat, ab, ptr_kind, &ad));
  FIT_TRY(stage_in(p, &p->in_c, carrier, fb, ptr_kind, &cd));
  if (!ad) {
    API_CHECK(p->M >= p->nd, FIT_ERR_ARG, "self-advection needs >= nd components (pass advecting_hat)");
    ad = ud;
  }
  if (!cd) cd = ud;
  FIT_TRY(ensure_shells(p, edges, n_edges, dims_mask, coord_f32));
  const int nsh = p->nsh;
  FIT_TRY(ensure(p, &p->outd, sizeof(double) * (nsh + 1)));
  double* Td = (double*)p->outd.p;
  if (p->prec == 64) {
    FIT_TRY(nonlinear_half<double>(p, ud, ad, 0, false));
    FIT_TRY(carrier_and_bin_setup<double>(p, cd, invariant));
    FIT_TRY(bin_into<double>(p, p->nh.p, 0, 1, p->ceff.p, Td));
  } else if (fz_box_ok(p)) {   // FP32 cubic 3D of a fused size: the nonlinear term on the live box
    FIT_TRY(s2s_box_flux(p, ud, ad, cd, invariant, Td));
    FIT_TRY(s2s_check(p));
  } else {
    FIT_TRY(nonlinear_half<float>(p, ud, ad, 0, false));
    FIT_TRY(carrier_and_bin_setup<float>(p, cd, invariant));
    FIT_TRY(bin_into<float>(p, p->nh.p, 0, 1, p->ceff.p, Td));
  }
  std::vector<double> h(nsh), pi(nsh);
  FIT_CUDA_CHECK(cudaMemcpyAsync(h.data(), Td, sizeof(double) * nsh, cudaMemcpyDeviceToHost, p->stream));
  FIT_TRY(sync_plan(p));
  double acc = 0.0;
  for (int n = 0; n < nsh; ++n) {   // Pi = +cumsum(T) (src/SpectralFlux.jl:176)
    acc += h[n];
    pi[n] = acc;
  }
  if (ptr_kind == FIT_PTR_DEVICE) {
    FIT_CUDA_CHECK(cudaMemcpyAsync(T, h.data(), sizeof(double) * nsh, cudaMemcpyHostToDevice, p->stream));
    if (Pi) FIT_CUDA_CHECK(cudaMemcpyAsync(Pi, pi.data(), sizeof(double) * nsh, cudaMemcpyHostToDevice, p->stream));
    return sync_plan(p);
  }
  memcpy(T, h.data(), sizeof(double) * nsh);
  if (Pi) memcpy(Pi, pi.data(), sizeof(double) * nsh);
  return FIT_OK;
}

// Inputs of a shell-to-shell call on the device (the batched form on a 2/3 plan copies only the
// kept box of host inputs).
static int s2s_stage(fit_plan* p, const void* u_hat, const void* adv_hat, int invariant, int mode, int ptr_kind,
                     const void** ud, const void** ad) {
  FIT_TRY(check_invariant(p, invariant, p->M));
  API_CHECK(mode == FIT_S2S_PLAIN || mode == FIT_S2S_BATCHED, FIT_ERR_ARG, "unknown shell-to-shell mode %d", mode);
  const size_t fb = cbytes(p) * p->g.Ntot * p->M, ab = cbytes(p) * p->g.Ntot * p->Dadv;
  p->kept_src = nullptr;
  if (mode == FIT_S2S_BATCHED && ptr_kind != FIT_PTR_DEVICE && s2s_reads_kept_box(p)) {
    FIT_TRY(stage_in_kept_box(p, &p->in_u, u_hat, fb, p->M, ud, true));
    FIT_TRY(stage_in_kept_box(p, &p->in_a, adv_hat, ab, p->Dadv, ad));
  } else {
    FIT_TRY(stage_in(p, &p->in_u, u_hat, fb, ptr_kind, ud));
    FIT_TRY(stage_in(p, &p->in_a, adv_hat, ab, ptr_kind, ad));
  }
  if (!*ad) {
    API_CHECK(p->M >= p->nd, FIT_ERR_ARG, "self-advection needs >= nd components (pass advecting_hat)");
    *ad = *ud;
  }
  return FIT_OK;
}

// T(n,m), net and max|T+T'| once the inputs are staged and the plan's shell table is set.
static int s2s_run(fit_plan* p, const void* ud, const void* ad, int invariant, int mode, int verify,
                   double* T_colmajor, double* net, double* max_asym, int ptr_kind) {
  const int nsh = p->nsh;
  FIT_TRY(ensure(p, &p->outd, sizeof(double) * (size_t)nsh * nsh));
  double* Td = (double*)p->outd.p;
  FIT_CUDA_CHECK(cudaMemsetAsync(Td, 0, sizeof(double) * (size_t)nsh * nsh, p->stream));
  if (mode == FIT_S2S_BATCHED) {
    const int rc = s2s_batched(p, ud, ad, invariant, Td);
    p->kept_src = nullptr;   // read (or abandoned) by this call
    FIT_TRY(rc);
    FIT_TRY(s2s_check(p));
  } else if (p->prec == 64) {
    FIT_TRY(carrier_and_bin_setup<double>(p, ud, invariant));
    for (int m = 1; m <= nsh; ++m) {
      FIT_TRY(nonlinear_half<double>(p, ud, ad, m, m > 1));
      FIT_TRY(bin_into<double>(p, p->nh.p, 0, 1, p->ceff.p, Td + (size_t)(m - 1) * nsh));
    }
  } else {
    FIT_TRY(carrier_and_bin_setup<float>(p, ud, invariant));
    for (int m = 1; m <= nsh; ++m) {
      FIT_TRY(nonlinear_half<float>(p, ud, ad, m, m > 1));
      FIT_TRY(bin_into<float>(p, p->nh.p, 0, 1, p->ceff.p, Td + (size_t)(m - 1) * nsh));
    }
  }
  std::vector<double> h((size_t)nsh * nsh), nt(nsh);
  FIT_CUDA_CHECK(cudaMemcpyAsync(h.data(), Td, sizeof(double) * h.size(), cudaMemcpyDeviceToHost, p->stream));
  FIT_TRY(sync_plan(p));
  double asym = 0.0;
  for (int n = 0; n < nsh; ++n) {   // net_transfer and max|T+T'| (ext/FlowInvariantTransferFFTWExt.jl:277-292)
    double s = 0.0;
    for (int m = 0; m < nsh; ++m) {
      s += h[n + (size_t)nsh * m];
      const double a = fabs(h[n + (size_t)nsh * m] + h[m + (size_t)nsh * n]);
      if (a > asym) asym = a;
    }
    nt[n] = s;
  }
  if (!verify) asym = NAN;
  if (ptr_kind == FIT_PTR_DEVICE) {
    FIT_CUDA_CHECK(cudaMemcpyAsync(T_colmajor, Td, sizeof(double) * h.size(), cudaMemcpyDeviceToDevice, p->stream));
    if (net) FIT_CUDA_CHECK(cudaMemcpyAsync(net, nt.data(), sizeof(double) * nsh, cudaMemcpyHostToDevice, p->stream));
    if (max_asym) FIT_CUDA_CHECK(cudaMemcpyAsync(max_asym, &asym, sizeof(double), cudaMemcpyHostToDevice, p->stream));
    return sync_plan(p);
  }
  memcpy(T_colmajor, h.data(), sizeof(double) * h.size());
  if (net) memcpy(net, nt.data(), sizeof(double) * nsh);
  if (max_asym) *max_asym = asym;
  return FIT_OK;
}

int fit_shell_to_shell(fit_plan* p, const void* u_hat, const void* adv_hat, const double* edges, int n_edges,
                       uint32_t dims_mask, int coord_f32, int invariant, int mode, int verify, double* T_colmajor,
                       double* net, double* max_asym, int ptr_kind) {
  API_CHECK(p != nullptr && u_hat != nullptr && T_colmajor != nullptr, FIT_ERR_ARG, "NULL argument");
  const void *ud, *ad;
  FIT_TRY(s2s_stage(p, u_hat, adv_hat, invariant, mode, ptr_kind, &ud, &ad));
  FIT_TRY(ensure_shells(p, edges, n_edges, dims_mask, coord_f32));
  return s2s_run(p, ud, ad, invariant, mode, verify, T_colmajor, net, max_asym, ptr_kind);
}

// Host shell index -> uint16 table, validated, split over up to 32 threads; *same tells whether the
// table equals prev (NULL: no previous table). Returns the lowest bad position, or -1.
static long index_to_table(const int64_t* idx, long n, int nsh, uint16_t* out, const uint16_t* prev, bool* same) {
  const long cores = (long)std::thread::hardware_concurrency();
  const int nthr = (int)(n < (1L << 20) ? 1 : (cores < 1 ? 1 : (cores > 32 ? 32 : cores)));
  std::vector<long> bad((size_t)nthr, -1);
  std::vector<char> eq((size_t)nthr, prev != nullptr);
  auto work = [&](int t) {
    const long a = n * t / nthr, b = n * (t + 1) / nthr;
    bool e = prev != nullptr;
    for (long i = a; i < b; ++i) {
      const int64_t v = idx[i];
      if (v < 0 || v > nsh) {
        bad[(size_t)t] = i;
        return;
      }
      out[i] = (uint16_t)v;
      e = e && prev[i] == out[i];
    }
    eq[(size_t)t] = e;
  };
  std::vector<std::thread> th;
  for (int t = 1; t < nthr; ++t) th.emplace_back(work, t);
  work(0);
  for (auto& x : th) x.join();
  *same = prev != nullptr;
  for (int t = 0; t < nthr; ++t) {
    if (bad[(size_t)t] >= 0) return bad[(size_t)t];
    *same = *same && eq[(size_t)t];
  }
  return -1;
}

// Installs a caller's shell index. A call whose index equals the installed one changes nothing, so
// a caller that rebuilds the same index on every call (the reference makes a new workspace per
// call) keeps the batched form's captured graph.
int fit_set_shell_index(fit_plan* p, const int64_t* shell_idx, int n_shells, int ptr_kind) {
  API_CHECK(p != nullptr && shell_idx != nullptr, FIT_ERR_ARG, "NULL argument");
  API_CHECK(n_shells >= 1 && n_shells <= 65535, FIT_ERR_ARG, "n_shells must be in 1..65535 (got %d)", n_shells);
  const long n = p->g.Ntot;
  const bool installed = p->cached_f32 == -2 && p->nsh == n_shells && p->shell_full.p != nullptr;
  bool changed = true;
  if (ptr_kind == FIT_PTR_DEVICE) {
    FIT_TRY(ensure(p, &p->shell_full, sizeof(uint16_t) * n));
    FIT_TRY(ensure(p, &p->flag, 16));
    FIT_CUDA_CHECK(cudaMemsetAsync(p->flag.p, 0xff, sizeof(unsigned long long), p->stream));
    FIT_CUDA_CHECK(cudaMemsetAsync((char*)p->flag.p + 8, 0, sizeof(unsigned), p->stream));
    FIT_TRY(shell_table_from_i64(p->g, shell_idx, n_shells, (uint16_t*)p->shell_full.p,
                                 (unsigned long long*)p->flag.p, (unsigned*)((char*)p->flag.p + 8), p->stream));
    unsigned long long h[2] = {0, 0};
    FIT_CUDA_CHECK(cudaMemcpyAsync(h, p->flag.p, 16, cudaMemcpyDeviceToHost, p->stream));
    FIT_TRY(sync_plan(p));
    p->idx_host.clear();
    if (h[0] != ~0ull) {
      p->cached_edges.clear();   // the table is partly written: no cache key may match it
      p->cached_f32 = -3;
      p->shell_gen++;
      fit_set_error("shell index at linear position %llu is outside [0, %d]", h[0], n_shells);
      return FIT_ERR_ARG;
    }
    changed = (unsigned)h[1] != 0u;
  } else {
    std::vector<uint16_t> t((size_t)n);
    bool same = false;
    const long bad = index_to_table(shell_idx, n, n_shells, t.data(),
                                    installed && p->idx_host.size() == (size_t)n ? p->idx_host.data() : nullptr,
                                    &same);
    API_CHECK(bad < 0, FIT_ERR_ARG, "shell index %lld at linear position %ld is outside [0, %d]",
              (long long)shell_idx[bad < 0 ? 0 : bad], bad, n_shells);
    if (same) {
      changed = false;
    } else {
      FIT_TRY(ensure(p, &p->shell_full, sizeof(uint16_t) * n));
      FIT_CUDA_CHECK(cudaMemcpyAsync(p->shell_full.p, t.data(), sizeof(uint16_t) * n, cudaMemcpyHostToDevice,
                                     p->stream));
      FIT_TRY(sync_plan(p));
      p->idx_host.swap(t);
    }
  }
  if (installed && !changed) return FIT_OK;
  p->cached_edges.clear();
  p->cached_dims = 0;
  p->cached_f32 = -2;
  p->nsh = n_shells;
  p->shell_gen++;
  return FIT_OK;
}

int fit_shell_to_shell_indexed(fit_plan* p, const void* u_hat, const void* adv_hat, int invariant, int mode,
                               int verify, double* T_colmajor, double* net, double* max_asym, int ptr_kind) {
  API_CHECK(p != nullptr && u_hat != nullptr && T_colmajor != nullptr, FIT_ERR_ARG, "NULL argument");
  API_CHECK(p->cached_f32 == -2 && p->nsh > 0, FIT_ERR_STATE,
            "no shell index is installed on this plan (fit_set_shell_index, or a later call with shell edges "
            "replaced it)");
  const void *ud, *ad;
  FIT_TRY(s2s_stage(p, u_hat, adv_hat, invariant, mode, ptr_kind, &ud, &ad));
  return s2s_run(p, ud, ad, invariant, mode, verify, T_colmajor, net, max_asym, ptr_kind);
}

int fit_helical_decompose(fit_plan* p, const void* u_hat, void* up, void* um, int ptr_kind) {
  API_CHECK(p != nullptr && u_hat != nullptr && up != nullptr && um != nullptr, FIT_ERR_ARG, "NULL argument");
  API_CHECK(p->nd == 3, FIT_ERR_ARG, "HelicalDecomposition is defined in 3D only (got nd=%d).", p->nd);
  API_CHECK(p->M >= 3, FIT_ERR_ARG, "HelicalDecomposition needs >=3 velocity components (got D=%d).", p->M);
  const size_t fb = cbytes(p) * p->g.Ntot * 3;
  const void* ud;
  FIT_TRY(stage_in(p, &p->in_u, u_hat, cbytes(p) * p->g.Ntot * p->M, ptr_kind, &ud));
  void *a = up, *b = um;
  if (ptr_kind != FIT_PTR_DEVICE) {
    FIT_TRY(ensure(p, &p->out_c, fb));
    FIT_TRY(ensure(p, &p->out_c2, fb));
    a = p->out_c.p;
    b = p->out_c2.p;
  }
  FIT_TRY(helical_split(p->g, p->kt, ud, p->io_f64, a, b, p->stream));
  if (ptr_kind != FIT_PTR_DEVICE) {
    FIT_TRY(copy_out(p, up, a, fb, ptr_kind));
    FIT_TRY(copy_out(p, um, b, fb, ptr_kind));
  }
  return sync_plan(p);
}

int fit_toroidal_poloidal_decompose(fit_plan* p, const void* u_hat, void* tor, void* pol, int ptr_kind) {
  API_CHECK(p != nullptr && u_hat != nullptr && tor != nullptr && pol != nullptr, FIT_ERR_ARG, "NULL argument");
  API_CHECK(p->nd == 3, FIT_ERR_ARG, "ToroidalPoloidalDecomposition is defined in 3D only (got nd=%d).", p->nd);
  API_CHECK(p->M >= 3, FIT_ERR_ARG, "ToroidalPoloidalDecomposition needs >=3 velocity components (got D=%d).", p->M);
  const size_t fb = cbytes(p) * p->g.Ntot * 3;
  const void* ud;
  FIT_TRY(stage_in(p, &p->in_u, u_hat, cbytes(p) * p->g.Ntot * p->M, ptr_kind, &ud));
  void *a = tor, *b = pol;
  if (ptr_kind != FIT_PTR_DEVICE) {
    FIT_TRY(ensure(p, &p->out_c, fb));
    FIT_TRY(ensure(p, &p->out_c2, fb));
    a = p->out_c.p;
    b = p->out_c2.p;
  }
  FIT_TRY(toroidal_split(p->g, p->kt, ud, p->io_f64, a, b, p->stream));
  if (ptr_kind != FIT_PTR_DEVICE) {
    FIT_TRY(copy_out(p, tor, a, fb, ptr_kind));
    FIT_TRY(copy_out(p, pol, b, fb, ptr_kind));
  }
  return sync_plan(p);
}

int fit_helmholtz_decompose(fit_plan* p, const void* u_hat, void* ur, void* udv, int ptr_kind) {
  API_CHECK(p != nullptr && u_hat != nullptr && ur != nullptr && udv != nullptr, FIT_ERR_ARG, "NULL argument");
  API_CHECK(p->nd == 2 && p->M == 2, FIT_ERR_ARG, "Helmholtz decomposition currently supports 2D fields only.");
  const size_t fb = cbytes(p) * p->g.Ntot * 2;
  const void* ud;
  FIT_TRY(stage_in(p, &p->in_u, u_hat, fb, ptr_kind, &ud));
  void *a = ur, *b = udv;
  if (ptr_kind != FIT_PTR_DEVICE) {
    FIT_TRY(ensure(p, &p->out_c, fb));
    FIT_TRY(ensure(p, &p->out_c2, fb));
    a = p->out_c.p;
    b = p->out_c2.p;
  }
  FIT_TRY(helmholtz_split(p->g, p->kt, ud, p->io_f64, a, b, p->stream));
  if (ptr_kind != FIT_PTR_DEVICE) {
    FIT_TRY(copy_out(p, ur, a, fb, ptr_kind));
    FIT_TRY(copy_out(p, udv, b, fb, ptr_kind));
  }
  return sync_plan(p);
}

int fit_partial_fluxes(fit_plan* p, const void* u_hat, int decomposition, int invariant, const double* edges,
                       int n_edges, uint32_t dims_mask, int coord_f32, double* T_channels, int ptr_kind) {
  API_CHECK(p != nullptr && u_hat != nullptr && T_channels != nullptr, FIT_ERR_ARG, "NULL argument");
  API_CHECK(decomposition == FIT_DECOMP_HELICAL || decomposition == FIT_DECOMP_HELMHOLTZ ||
                decomposition == FIT_DECOMP_TOROIDAL_POLOIDAL,
            FIT_ERR_ARG, "calculate_partial_fluxes needs a decomposition that splits u into >=2 named components");
  API_CHECK(p->M == p->nd && p->Dadv == p->nd, FIT_ERR_ARG, "partial fluxes need an nd-component velocity plan");
  FIT_TRY(check_invariant(p, invariant, p->M));
  const size_t fb = cbytes(p) * p->g.Ntot * p->M;
  const void* ud;
  FIT_TRY(stage_in(p, &p->in_u, u_hat, fb, ptr_kind, &ud));
  FIT_TRY(ensure(p, &p->out_c, fb));
  FIT_TRY(ensure(p, &p->out_c2, fb));
  if (decomposition == FIT_DECOMP_HELICAL) FIT_TRY(helical_split(p->g, p->kt, ud, p->io_f64, p->out_c.p, p->out_c2.p, p->stream));
  else if (decomposition == FIT_DECOMP_TOROIDAL_POLOIDAL)
    FIT_TRY(toroidal_split(p->g, p->kt, ud, p->io_f64, p->out_c.p, p->out_c2.p, p->stream));
  else FIT_TRY(helmholtz_split(p->g, p->kt, ud, p->io_f64, p->out_c.p, p->out_c2.p, p->stream));
  const void* comp[2] = {p->out_c.p, p->out_c2.p};
  FIT_TRY(ensure_shells(p, edges, n_edges, dims_mask, coord_f32));
  const int nsh = p->nsh;
  FIT_TRY(ensure(p, &p->outd, sizeof(double) * 8 * nsh));
  double* Td = (double*)p->outd.p;
  const size_t vb = p->prec == 64 ? 16 : 8;
  // effective carriers of both components (3 fields each) at ceff[0..2] and ceff[3..5]
  FIT_TRY(ensure(p, &p->ceff, vb * 6 * p->g.Mhalf));
  FIT_TRY(ensure(p, &p->seff, sizeof(uint16_t) * p->g.Mhalf));
  for (int sk = 0; sk < 2; ++sk) {
    void* cptr = (char*)p->ceff.p + vb * 3 * p->g.Mhalf * sk;
    if (p->prec == 64)
      FIT_TRY(effective_carrier<double>(p->g, p->kt, comp[sk], p->io_f64, p->g.Ntot, p->M, invariant, p->dealias == 1,
                                        (const uint16_t*)p->shell_full.p, (double2*)cptr, p->M, (uint16_t*)p->seff.p,
                                        p->stream));
    else
      FIT_TRY(effective_carrier<float>(p->g, p->kt, comp[sk], p->io_f64, p->g.Ntot, p->M, invariant, p->dealias == 1,
                                       (const uint16_t*)p->shell_full.p, (float2*)cptr, p->M, (uint16_t*)p->seff.p,
                                       p->stream));
  }
  for (int sp = 0; sp < 2; ++sp)
    for (int sq = 0; sq < 2; ++sq) {   // N = (u_sp . grad) u_sq  (src/SpectralFlux.jl:275)
      if (p->prec == 64) FIT_TRY(nonlinear_half<double>(p, comp[sq], comp[sp], 0, false));
      else FIT_TRY(nonlinear_half<float>(p, comp[sq], comp[sp], 0, false));
      for (int sk = 0; sk < 2; ++sk) {
        const void* cptr = (const char*)p->ceff.p + vb * 3 * p->g.Mhalf * sk;
        double* dst = Td + (size_t)(sk * 4 + sp * 2 + sq) * nsh;
        if (p->prec == 64) FIT_TRY(bin_into<double>(p, p->nh.p, 0, 1, cptr, dst));
        else FIT_TRY(bin_into<float>(p, p->nh.p, 0, 1, cptr, dst));
      }
    }
  FIT_TRY(copy_out(p, T_channels, Td, sizeof(double) * 8 * nsh, ptr_kind));
  return sync_plan(p);
}

int fit_mode_to_mode(fit_plan* p, const void* u_hat, const void* adv_hat, int invariant, int fp64_products, double* S,
                     double* net, int ptr_kind) {
  API_CHECK(p != nullptr && u_hat != nullptr && S != nullptr, FIT_ERR_ARG, "NULL argument");
  FIT_TRY(check_invariant(p, invariant, p->M));
  API_CHECK(p->dealias != 2, FIT_ERR_ARG, "mode-to-mode triads support NoDealiasing and OrszagTwoThirds");
  const size_t fb = cbytes(p) * p->g.Ntot * p->M, ab = cbytes(p) * p->g.Ntot * p->Dadv;
  const void *ud, *ad;
  FIT_TRY(stage_in(p, &p->in_u, u_hat, fb, ptr_kind, &ud));
  FIT_TRY(stage_in(p, &p->in_a, adv_hat, ab, ptr_kind, &ad));
  if (!ad) {
    API_CHECK(p->M >= p->nd, FIT_ERR_ARG, "self-advection needs >= nd components (pass advecting_hat)");
    ad = ud;
  }
  const long nm = p->g.Ntot;
  const size_t sb = sizeof(double) * (size_t)nm * nm;
  double *Sd = S, *nd_ = net;
  if (ptr_kind != FIT_PTR_DEVICE) {
    FIT_TRY(ensure(p, &p->out_c, sb));
    FIT_TRY(ensure(p, &p->outd, sizeof(double) * nm));
    Sd = (double*)p->out_c.p;
    nd_ = (double*)p->outd.p;
  } else if (!nd_) {
    FIT_TRY(ensure(p, &p->outd, sizeof(double) * nm));
    nd_ = (double*)p->outd.p;
  }
  FIT_TRY(triad_m2m(p, ud, ad, invariant, fp64_products, Sd, nd_));
  if (ptr_kind != FIT_PTR_DEVICE) {
    FIT_TRY(copy_out(p, S, Sd, sb, ptr_kind));
    FIT_TRY(copy_out(p, net, nd_, sizeof(double) * nm, ptr_kind));
  }
  return sync_plan(p);
}

}  // extern "C"
