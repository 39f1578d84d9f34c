// Batched shell-to-shell transfer: every mediator shell's nonlinear term (u . grad) u_m
// (ext/FlowInvariantTransferFFTWExt.jl:245-275) evaluated in batches of mediators with one
// binning launch per batch, the whole sequence captured once into a CUDA graph and replayed.
//
// Shells with no retained mode contribute an exactly-zero column (the reference transforms
// zero fields), so they are skipped. The advecting velocity is transformed once per call.
#include <string.h>

#include <vector>

#include "fit_plan.cuh"

namespace fit {

struct S2SState {
  cudaGraphExec_t exec = nullptr;
  long graph_launches = 0;
  const void* key_u = nullptr;
  const void* key_a = nullptr;
  int key_inv = -1;
  std::vector<double> key_edges;
  unsigned key_dims = 0;
  int key_f32 = -1;
  long key_gen = -1;
  const double* key_T = nullptr;
  std::vector<int> occ;   // retained modes per shell
  fit_dbuf occ_dev;
};

void s2s_free(fit_plan* p) {
  S2SState* s = (S2SState*)p->s2s;
  if (!s) return;
  if (s->exec) cudaGraphExecDestroy(s->exec);
  if (s->occ_dev.p) cudaFree(s->occ_dev.p);
  delete s;
  p->s2s = nullptr;
}

__global__ void k_occupancy(GridDesc g, const uint16_t* __restrict__ sh, int two_thirds, int* occ) {
  const long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (i >= g.Ntot) return;
  const int s = sh[i];
  if (!s) return;
  if (two_thirds) {
    int k[3];
    k[0] = (int)(i % g.N[0]);
    const long r = i / g.N[0];
    k[1] = (int)(r % g.N[1]);
    k[2] = (int)(r / g.N[1]);
    for (int d = 0; d < g.nd; ++d) {
      const int N = g.N[d];
      const int a = (k[d] <= N / 2) ? k[d] : N - k[d];
      if (a >= N / 3) return;
    }
  }
  atomicAdd(&occ[s - 1], 1);
}

template <typename T>
static int run_batched(fit_plan* p, S2SState* s, const void* ud, const void* ad, int inv, double* Td) {
  typedef typename Vec2<T>::t V;
  const GridDesc& g = p->g;
  const int nd = p->nd, M = p->M, nsh = p->nsh;
  // batch size: keep the per-batch workspace near 24 GB and at most 8 mediators
  const double per_med = (double)M * nd * (sizeof(V) * g.Mhalf + sizeof(T) * g.Mtot) +
                         (double)M * (sizeof(T) * g.Mtot + sizeof(V) * g.Mhalf);
  int B = (int)(24e9 / per_med);
  if (B > 8) B = 8;
  if (B < 1) B = 1;
  const long nfg = (long)M * nd;
  FIT_TRY(ensure(p, &p->hs, sizeof(V) * (nd + nfg * B) * g.Mhalf));
  FIT_TRY(ensure(p, &p->ph, sizeof(T) * (nd + nfg * B) * g.Mtot));
  FIT_TRY(ensure(p, &p->nph, sizeof(T) * M * B * g.Mtot));
  FIT_TRY(ensure(p, &p->nh, sizeof(V) * M * B * g.Mhalf));
  FIT_TRY(ensure(p, &p->ceff, sizeof(V) * 3 * g.Mhalf));
  FIT_TRY(ensure(p, &p->seff, sizeof(uint16_t) * g.Mhalf));
  const long cap = 2L * 152 * B * nsh;
  FIT_TRY(ensure(p, &p->partial, sizeof(double) * cap));
  V* hs = (V*)p->hs.p;
  T* ph = (T*)p->ph.p;
  FIT_TRY(effective_carrier<T>(g, p->kt, ud, p->io_f64, g.Ntot, M, inv, p->dealias == 1,
                               (const uint16_t*)p->shell_full.p, (V*)p->ceff.p, M, (uint16_t*)p->seff.p, p->stream));
  GatherArgs a;
  memset(&a, 0, sizeof(a));
  a.src[0] = ud;
  a.src[1] = ad;
  a.src_comp_stride[0] = g.Ntot;
  a.src_comp_stride[1] = g.Ntot;
  a.in_f64 = p->io_f64;
  a.two_thirds = p->dealias == 1;
  a.shell_full = (const uint16_t*)p->shell_full.p;
  a.scale = 1.0;
  const T inv_m = (T)(1.0 / (double)g.Mtot);
  a.nfields = nd;
  for (int j = 0; j < nd; ++j) a.f[j] = GatherField{1, j, -1, 0};
  FIT_TRY(gather_half<T>(g, p->kt, a, hs, p->stream));
  FIT_TRY(inverse_nd<T>(hs, ph, g, p->ax, nd, inv_m, p->stream));
  std::vector<int> meds;
  for (int m = 1; m <= nsh; ++m)
    if (s->occ[m - 1] > 0) meds.push_back(m);
  const double fs = g.padded ? (double)g.Mtot / ((double)g.Ntot * (double)g.Ntot) : 1.0 / (double)g.Ntot;
  V* hg = hs + (long)nd * g.Mhalf;
  T* pg = ph + (long)nd * g.Mtot;
  for (size_t b0 = 0; b0 < meds.size(); b0 += B) {
    const int nb = (int)((meds.size() - b0) < (size_t)B ? (meds.size() - b0) : (size_t)B);
    // gather nb * M * nd derivative fields, at most 16 per launch
    long fi = 0;
    std::vector<GatherField> all;
    for (int b = 0; b < nb; ++b)
      for (int c = 0; c < M; ++c)
        for (int j = 0; j < nd; ++j) all.push_back(GatherField{0, c, j, meds[b0 + b]});
    while (fi < (long)all.size()) {
      const int cnt = (int)(((long)all.size() - fi) < 16 ? ((long)all.size() - fi) : 16);
      a.nfields = cnt;
      for (int q = 0; q < cnt; ++q) a.f[q] = all[fi + q];
      FIT_TRY(gather_half<T>(g, p->kt, a, hg + fi * g.Mhalf, p->stream));
      fi += cnt;
    }
    FIT_TRY(inverse_nd<T>(hg, pg, g, p->ax, nfg * nb, inv_m, p->stream));
    for (int b = 0; b < nb; ++b)
      FIT_TRY(product<T>(ph, pg + (long)b * nfg * g.Mtot, (T*)p->nph.p + (long)b * M * g.Mtot, nd, M, g.Mtot,
                         p->stream));
    FIT_TRY(forward_nd<T>((const T*)p->nph.p, (V*)p->nh.p, g, p->ax, (long)M * nb, (T)fs, p->stream));
    // columns of consecutive mediators are contiguous in the column-major T
    int b = 0;
    while (b < nb) {
      int e = b + 1;
      while (e < nb && meds[b0 + e] == meds[b0 + e - 1] + 1) ++e;
      FIT_TRY(bin_density<T>(g, (const V*)p->nh.p + (long)b * M * g.Mhalf, (long)M * g.Mhalf, e - b,
                             (const V*)p->ceff.p, M, (const uint16_t*)p->seff.p, nsh, (double*)p->partial.p, cap,
                             Td + (long)(meds[b0 + b] - 1) * nsh, p->stream));
      b = e;
    }
  }
  return FIT_OK;
}

int s2s_batched(fit_plan* p, const void* ud, const void* ad, int inv, double* Td) {
  S2SState* s = (S2SState*)p->s2s;
  if (!s) {
    s = new S2SState();
    p->s2s = s;
  }
  // A captured graph bakes every pointer it touches: it is replayed only while the inputs, the
  // output, the shell set and every workspace allocation are unchanged.
  const bool same = s->key_u == ud && s->key_a == ad && s->key_inv == inv && s->key_edges == p->cached_edges &&
                    s->key_dims == p->cached_dims && s->key_f32 == p->cached_f32 && s->key_T == Td &&
                    s->key_gen == p->buf_gen;
  if (!same) {
    if (s->exec) cudaGraphExecDestroy(s->exec);
    s->exec = nullptr;
    // retained-mode occupancy of every shell
    FIT_TRY(ensure(p, &s->occ_dev, sizeof(int) * p->nsh));
    FIT_CUDA_CHECK(cudaMemsetAsync(s->occ_dev.p, 0, sizeof(int) * p->nsh, p->stream));
    k_occupancy<<<(unsigned)((p->g.Ntot + 255) / 256), 256, 0, p->stream>>>(
        p->g, (const uint16_t*)p->shell_full.p, p->dealias == 1, (int*)s->occ_dev.p);
    FIT_LAUNCH_CHECK();
    s->occ.assign(p->nsh, 0);
    FIT_CUDA_CHECK(cudaMemcpyAsync(s->occ.data(), s->occ_dev.p, sizeof(int) * p->nsh, cudaMemcpyDeviceToHost, p->stream));
    FIT_CUDA_CHECK(cudaStreamSynchronize(p->stream));
    // first call for this key: run eagerly (allocates the workspace, sets kernel attributes)
    const int rc = (p->prec == 64) ? run_batched<double>(p, s, ud, ad, inv, Td) : run_batched<float>(p, s, ud, ad, inv, Td);
    if (rc != FIT_OK) return rc;
    s->key_u = ud;
    s->key_a = ad;
    s->key_inv = inv;
    s->key_edges = p->cached_edges;
    s->key_dims = p->cached_dims;
    s->key_f32 = p->cached_f32;
    s->key_T = Td;
    s->key_gen = p->buf_gen;
    return FIT_OK;
  }
  if (fit_prof_on()) {   // per-launch events need eager launches
    return (p->prec == 64) ? run_batched<double>(p, s, ud, ad, inv, Td) : run_batched<float>(p, s, ud, ad, inv, Td);
  }
  if (s->exec) {
    FIT_CUDA_CHECK(cudaGraphLaunch(s->exec, p->stream));
    fit_count_launches(s->graph_launches);
    return FIT_OK;
  }
  // second call with the same key: capture the sequence, then replay it from now on
  cudaGraph_t graph = nullptr;
  FIT_CUDA_CHECK(cudaStreamBeginCapture(p->stream, cudaStreamCaptureModeThreadLocal));
  const long before = fit_launch_total();
  int rc = (p->prec == 64) ? run_batched<double>(p, s, ud, ad, inv, Td) : run_batched<float>(p, s, ud, ad, inv, Td);
  const long captured = fit_launch_total() - before;
  cudaError_t ce = cudaStreamEndCapture(p->stream, &graph);
  fit_count_launches(-captured);
  if (rc != FIT_OK) {
    if (graph) cudaGraphDestroy(graph);
    return rc;
  }
  if (ce != cudaSuccess) {
    fit_set_error("stream capture failed: %s", cudaGetErrorString(ce));
    return FIT_ERR_CUDA;
  }
  if (p->buf_gen != s->key_gen) {   // a workspace moved while capturing: do not keep the graph
    cudaGraphDestroy(graph);
    fit_set_error("workspace reallocated during capture");
    return FIT_ERR_STATE;
  }
  cudaError_t ie = cudaGraphInstantiate(&s->exec, graph, 0);
  cudaGraphDestroy(graph);
  if (ie != cudaSuccess) {
    s->exec = nullptr;
    fit_set_error("graph instantiate failed: %s", cudaGetErrorString(ie));
    return FIT_ERR_CUDA;
  }
  s->graph_launches = captured;
  FIT_CUDA_CHECK(cudaGraphLaunch(s->exec, p->stream));
  fit_count_launches(captured);
  return FIT_OK;
}

}  // namespace fit
