// Batched partial fluxes: the 8 channels Pi^{s_k s_p s_q}(K) (src/SpectralFlux.jl:240-285) of one
// or several invariants (kinetic energy, helicity) from ONE pass over the components, replayed as
// one CUDA graph launch.
//
// The reference computes one nonlinear term N = (u_sp . grad) u_sq per (sp, sq) pair and per
// invariant call. Here the two components' velocities (2 nd fields) and gradients (2 nd^2 fields)
// are transformed to physical space once; each of the four (sp, sq) products is then one product
// kernel and one forward transform, and its N̂ is binned against the effective carriers of every
// requested invariant and component s_k. For nd = 3 this is 24 inverse + 12 forward field
// transforms for any number of invariants, against 4 x (3 + 9) + 4 x 3 = 60 per invariant.
// The first call for a key runs eagerly (allocation, autotuning if enabled); the second captures
// the sequence into a graph; later calls replay it.
#include <string.h>

#include <vector>

#include "fit_fused_impl.cuh"
#include "fit_gb300.h"
#include "fit_plan.cuh"

namespace fit {

// live-box pipeline pieces (fit_s2s.cu)
bool fz_box_ok(const fit_plan* p);
void fz_box_dims(const fit_plan* p, FzArgs* a);
int fz_box_setup(fit_plan* p, const FzArgs& a, const void* F, int inv, float2* H, float2* Ceff, uint16_t* seff,
                 uint16_t* sb, int inv2, float2* Ceff2);
int fz_box_kd(fit_plan* p, const FzArgs& a, float* kd);
int fz_box_velocity(fit_plan* p, const FzArgs& a, const float2* H, float2* bufZ, float2* bufY, float* U);
int fz_box_terms(fit_plan* p, const FzArgs& a, const float2* H, const float* kd, const float* U, float2* bufA,
                 float2* bufB, float2* Nout, int* err);

struct PartialState {
  fit_dbuf comp, ceff, phys, hs, nph, nh;
  // live-box form: H and carriers per component, velocities, scratch, the four terms, wait flag
  fit_dbuf bH, bC, bse, bsb, bkd, bU, bA, bB, bN, berr;
  int bkd_n = -1;
  cudaGraphExec_t exec = nullptr;
  long graph_launches = 0;
  // graph key
  const void* key_u = nullptr;
  int key_decomp = -1;
  std::vector<int> key_inv;
  std::vector<double> key_edges;
  unsigned key_dims = 0;
  int key_f32 = -1;
  double* key_T = nullptr;
  long key_gen = -1;
  long key_sgen = -1;
  cudaStream_t key_stream = nullptr;
};

static int pbuf(fit_plan* p, fit_dbuf* b, size_t bytes) { return ensure(p, b, bytes); }

template <typename T>
static int run_partial(fit_plan* p, PartialState* s, const void* ud, int decomposition, const int* invs, int ninv,
                       double* Td) {
  typedef typename Vec2<T>::t V;
  const GridDesc& g = p->g;
  const int nd = p->nd, M = p->M;
  const size_t cb = (p->io_f64 ? 16 : 8) * (size_t)g.Ntot * M;
  FIT_TRY(pbuf(p, &s->comp, 2 * cb));
  void* comp[2] = {s->comp.p, (char*)s->comp.p + cb};
  if (decomposition == FIT_DECOMP_HELICAL) FIT_TRY(helical_split(g, p->kt, ud, p->io_f64, comp[0], comp[1], p->stream));
  else if (decomposition == FIT_DECOMP_TOROIDAL_POLOIDAL)
    FIT_TRY(toroidal_split(g, p->kt, ud, p->io_f64, comp[0], comp[1], p->stream));
  else FIT_TRY(helmholtz_split(g, p->kt, ud, p->io_f64, comp[0], comp[1], p->stream));
  // effective carriers: (invariant j, component sk) -> M fields each
  const size_t csz = sizeof(V) * (size_t)M * g.Mhalf;
  FIT_TRY(pbuf(p, &s->ceff, csz * 2 * ninv));
  FIT_TRY(ensure(p, &p->seff, sizeof(uint16_t) * g.Mhalf));
  for (int j = 0; j < ninv; ++j)
    for (int sk = 0; sk < 2; ++sk)
      FIT_TRY(effective_carrier<T>(g, p->kt, comp[sk], p->io_f64, g.Ntot, M, invs[j], p->dealias == 1,
                                   (const uint16_t*)p->shell_full.p, (V*)((char*)s->ceff.p + csz * (j * 2 + sk)), M,
                                   (uint16_t*)p->seff.p, p->stream));
  // physical fields: U[s] (nd each) then G[s] (M*nd each, component c*nd + j = d_j comp_s,c)
  const long nU = nd, nG = (long)M * nd, nf = 2 * (nU + nG);
  FIT_TRY(pbuf(p, &s->phys, sizeof(T) * nf * g.Mtot));
  const int chunk = 8;
  FIT_TRY(pbuf(p, &s->hs, sizeof(V) * chunk * g.Mhalf));
  GatherArgs a;
  memset(&a, 0, sizeof(a));
  a.src[0] = comp[0];
  a.src[1] = comp[1];
  a.src_comp_stride[0] = a.src_comp_stride[1] = g.Ntot;
  a.in_f64 = p->io_f64;
  a.two_thirds = p->dealias == 1;
  a.shell_full = (const uint16_t*)p->shell_full.p;
  a.scale = 1.0;
  std::vector<GatherField> all;
  for (int sc = 0; sc < 2; ++sc)
    for (int j = 0; j < nd; ++j) all.push_back(GatherField{sc, j, -1, 0, 0});
  for (int sc = 0; sc < 2; ++sc)
    for (int c = 0; c < M; ++c)
      for (int j = 0; j < nd; ++j) all.push_back(GatherField{sc, c, j, 0, 0});
  const T inv_m = (T)(1.0 / (double)g.Mtot);
  T* phys = (T*)s->phys.p;
  for (long f0 = 0; f0 < nf; f0 += chunk) {
    const int n = (int)((nf - f0) < chunk ? (nf - f0) : chunk);
    a.nfields = n;
    for (int i = 0; i < n; ++i) a.f[i] = all[f0 + i];
    FIT_TRY(gather_half<T>(g, p->kt, a, (V*)s->hs.p, p->stream));
    FIT_TRY(inverse_nd<T>((V*)s->hs.p, phys + f0 * g.Mtot, g, p->ax, n, inv_m, p->stream));
  }
  FIT_TRY(pbuf(p, &s->nph, sizeof(T) * M * g.Mtot));
  FIT_TRY(pbuf(p, &s->nh, sizeof(V) * M * g.Mhalf));
  const double fs = g.padded ? (double)g.Mtot / ((double)g.Ntot * (double)g.Ntot) : 1.0 / (double)g.Ntot;
  const int nsh = p->nsh;
  for (int sp = 0; sp < 2; ++sp)
    for (int sq = 0; sq < 2; ++sq) {   // N = (u_sp . grad) u_sq  (src/SpectralFlux.jl:275)
      const T* U = phys + (long)sp * nU * g.Mtot;
      const T* G = phys + (2 * nU + (long)sq * nG) * g.Mtot;
      FIT_TRY(product<T>(U, G, (T*)s->nph.p, nd, M, g.Mtot, p->stream));
      FIT_TRY(forward_nd<T>((const T*)s->nph.p, (V*)s->nh.p, g, p->ax, M, (T)fs, p->stream));
      // every (invariant, s_k) carrier set against this N̂ in one binning pass
      BinOut o;
      for (int j = 0; j < ninv; ++j)
        for (int sk = 0; sk < 2; ++sk) o.p[j * 2 + sk] = Td + ((size_t)j * 8 + sk * 4 + sp * 2 + sq) * nsh;
      const long cap = 2L * 152 * 2 * ninv * nsh;
      FIT_TRY(ensure(p, &p->partial, sizeof(double) * cap));
      FIT_TRY(bin_density_multi<T>(g, (const V*)s->nh.p, 0, 1, (const V*)s->ceff.p, (long)M * g.Mhalf, 2 * ninv, M,
                                   (const uint16_t*)p->seff.p, nsh, (double*)p->partial.p, cap, o, p->stream));
    }
  return FIT_OK;
}

// Live-box form for FP32 cubic 3D plans with a fused transform size: each component s gets H_s and
// its carriers on the live box (k_fz_setup) and its velocity in physical space; the four terms
// N = (u_sp . grad) u_sq run as one batch of four whole-box "mediators" through the fused passes
// (z pass of H_sq, y pass, x pass with u_sp, forward y and z), and one binning pass takes all four
// against every (invariant, s_k) carrier set.
static int run_partial_box(fit_plan* p, PartialState* s, const void* ud, int decomposition, const int* invs,
                           int ninv, double* Td) {
  const GridDesc& g = p->g;
  const size_t cb = (p->io_f64 ? 16 : 8) * (size_t)g.Ntot * 3;
  FIT_TRY(pbuf(p, &s->comp, 2 * cb));
  void* comp[2] = {s->comp.p, (char*)s->comp.p + cb};
  if (decomposition == FIT_DECOMP_HELICAL) FIT_TRY(helical_split(g, p->kt, ud, p->io_f64, comp[0], comp[1], p->stream,
                                                             p->dealias == 1));
  else if (decomposition == FIT_DECOMP_TOROIDAL_POLOIDAL)
    FIT_TRY(toroidal_split(g, p->kt, ud, p->io_f64, comp[0], comp[1], p->stream, p->dealias == 1));
  else FIT_TRY(helmholtz_split(g, p->kt, ud, p->io_f64, comp[0], comp[1], p->stream));
  FzArgs a;
  fz_box_dims(p, &a);
  const long BL = (long)a.KY * a.P1;   // live-box modes per field
  const double M = g.M[0];
  const double perA = 6.0 * M * a.P1S > 3.0 * a.L * a.KXS ? 6.0 * M * a.P1S : 3.0 * a.L * a.KXS;
  const double perB = 9.0 * a.L * a.KXS > 3.0 * M * a.P1S ? 9.0 * a.L * a.KXS : 3.0 * M * a.P1S;
  FIT_TRY(pbuf(p, &s->bH, sizeof(float2) * 6 * BL));
  FIT_TRY(pbuf(p, &s->bC, sizeof(float2) * 3 * BL * 2 * ninv));
  FIT_TRY(pbuf(p, &s->bse, sizeof(uint16_t) * BL));
  FIT_TRY(pbuf(p, &s->bsb, sizeof(uint16_t) * BL));
  FIT_TRY(pbuf(p, &s->bkd, sizeof(float) * a.KY));
  FIT_TRY(pbuf(p, &s->bU, sizeof(float) * 6 * g.Mtot));
  FIT_TRY(pbuf(p, &s->bA, (size_t)(8.0 * perA * 4)));
  FIT_TRY(pbuf(p, &s->bB, (size_t)(8.0 * perB * 4)));
  FIT_TRY(pbuf(p, &s->bN, sizeof(float2) * 12 * BL));
  if (!s->berr.p) {   // wait-timeout flag of the bulk-copy x pass (cleared once, outside capture)
    FIT_TRY(pbuf(p, &s->berr, sizeof(int)));
    FIT_CUDA_CHECK(cudaMemset(s->berr.p, 0, sizeof(int)));
  }
  if (s->bkd_n != a.KY) {   // never during a capture: the first call for a key runs eagerly
    FIT_TRY(fz_box_kd(p, a, (float*)s->bkd.p));
    s->bkd_n = a.KY;
  }
  float2* H = (float2*)s->bH.p;
  float2* Cf = (float2*)s->bC.p;
  for (int sk = 0; sk < 2; ++sk)   // H_sk and the carriers of two invariants per pass over the field
    for (int j = 0; j < ninv; j += 2)
      FIT_TRY(fz_box_setup(p, a, comp[sk], invs[j], H + (long)sk * 3 * BL, Cf + (long)(j * 2 + sk) * 3 * BL,
                           (uint16_t*)s->bse.p, (uint16_t*)s->bsb.p, j + 1 < ninv ? invs[j + 1] : -1,
                           j + 1 < ninv ? Cf + (long)((j + 1) * 2 + sk) * 3 * BL : nullptr));
  float* U = (float*)s->bU.p;
  for (int sp = 0; sp < 2; ++sp)
    FIT_TRY(fz_box_velocity(p, a, H + (long)sp * 3 * BL, (float2*)s->bA.p, (float2*)s->bB.p,
                            U + (long)sp * 3 * g.Mtot));
  a.nb = 4;
  for (int b = 0; b < 4; ++b) {   // term b = (sp, sq): N = (u_sp . grad) u_sq  (src/SpectralFlux.jl:275)
    a.uidx[b] = b >> 1;
    a.hidx[b] = b & 1;
    a.ext[b][0] = a.ext[b][1] = a.ext[b][2] = (short)a.K;
  }
  float2* Nb = (float2*)s->bN.p;
  FIT_TRY(fz_box_terms(p, a, H, (const float*)s->bkd.p, U, (float2*)s->bA.p, (float2*)s->bB.p, Nb,
                       (int*)s->berr.p));
  // all four terms against every (invariant, s_k) carrier set in one binning pass:
  // out.p[set][b * nsh + n] with set = j * 2 + sk lands at channel j * 8 + sk * 4 + b
  const int nsh = p->nsh;
  BinOut o;
  for (int j = 0; j < ninv; ++j)
    for (int sk = 0; sk < 2; ++sk) o.p[j * 2 + sk] = Td + ((size_t)j * 8 + sk * 4) * nsh;
  const long cap = 2L * 152 * 2 * ninv * 4 * nsh;
  FIT_TRY(ensure(p, &p->partial, sizeof(double) * cap));
  FIT_TRY(bin_density_multi<float>(g, Nb, 3 * BL, 4, Cf, 3 * BL, 2 * ninv, 3, (const uint16_t*)s->bse.p, nsh,
                                   (double*)p->partial.p, cap, o, p->stream, BL));
  return FIT_OK;
}

// A bounded wait inside the live-box x pass that gave up leaves its flag set: report it.
static int partial_box_check(fit_plan* p) {
  PartialState* s = (PartialState*)p->partial_state;
  if (!s || !s->berr.p) return FIT_OK;
  int h = 0;
  FIT_CUDA_CHECK(cudaMemcpyAsync(&h, s->berr.p, sizeof(int), cudaMemcpyDeviceToHost, p->stream));
  FIT_CUDA_CHECK(cudaStreamSynchronize(p->stream));
  if (h) {
    FIT_CUDA_CHECK(cudaMemset(s->berr.p, 0, sizeof(int)));
    fit_set_error("a bulk-copy wait timed out inside the fused partial-flux kernels");
    return FIT_ERR_STATE;
  }
  return FIT_OK;
}

static int run_any(fit_plan* p, PartialState* s, const void* ud, int dec, const int* invs, int ninv, double* Td) {
  if (fz_box_ok(p) && p->nd == 3 && ninv <= 4) return run_partial_box(p, s, ud, dec, invs, ninv, Td);
  return p->prec == 64 ? run_partial<double>(p, s, ud, dec, invs, ninv, Td)
                       : run_partial<float>(p, s, ud, dec, invs, ninv, Td);
}

static int partial_batched(fit_plan* p, const void* ud, int dec, const int* invs, int ninv, double* Td) {
  PartialState* s = (PartialState*)p->partial_state;
  if (!s) {
    s = new PartialState();
    p->partial_state = s;
  }
  std::vector<int> iv(invs, invs + ninv);
  const bool same = s->key_u == ud && s->key_decomp == dec && s->key_inv == iv && s->key_edges == p->cached_edges &&
                    s->key_dims == p->cached_dims && s->key_f32 == p->cached_f32 && s->key_T == Td &&
                    s->key_gen == p->buf_gen && s->key_stream == p->stream && s->key_sgen == p->shell_gen;
  if (!same) {
    if (s->exec) cudaGraphExecDestroy(s->exec);
    s->exec = nullptr;
    FIT_TRY(run_any(p, s, ud, dec, invs, ninv, Td));
    s->key_u = ud;
    s->key_decomp = dec;
    s->key_inv = iv;
    s->key_edges = p->cached_edges;
    s->key_dims = p->cached_dims;
    s->key_f32 = p->cached_f32;
    s->key_T = Td;
    s->key_gen = p->buf_gen;
    s->key_stream = p->stream;
    s->key_sgen = p->shell_gen;
    return FIT_OK;
  }
  // eager when profiling (per-launch events) or on the legacy default stream (not capturable)
  if (fit_prof_on() || p->stream == nullptr) return run_any(p, s, ud, dec, invs, ninv, Td);
  if (s->exec) {
    FIT_CUDA_CHECK(cudaGraphLaunch(s->exec, p->stream));
    fit_count_launches(s->graph_launches);
    return FIT_OK;
  }
  cudaGraph_t graph = nullptr;
  FIT_CUDA_CHECK(cudaStreamBeginCapture(p->stream, cudaStreamCaptureModeThreadLocal));
  const long before = fit_launch_total();
  int rc = run_any(p, s, ud, dec, invs, ninv, Td);
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
  if (p->buf_gen != s->key_gen) {
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

void partial_free(fit_plan* p) {
  PartialState* s = (PartialState*)p->partial_state;
  if (!s) return;
  if (s->exec) cudaGraphExecDestroy(s->exec);
  fit_dbuf* bufs[] = {&s->comp, &s->ceff, &s->phys, &s->hs, &s->nph, &s->nh, &s->bH, &s->bC,
                      &s->bse,  &s->bsb,  &s->bkd,  &s->bU, &s->bA,  &s->bB,  &s->bN, &s->berr};
  for (fit_dbuf* b : bufs) {
    if (b->p) {
      cudaFree(b->p);
      p->bytes -= b->cap;
    }
    b->p = nullptr;
    b->cap = 0;
  }
  delete s;
  p->partial_state = nullptr;
}

}  // namespace fit

using namespace fit;

extern "C" int fit_partial_fluxes_batched(fit_plan* p, const void* u_hat, int decomposition, const int* invariants,
                                          int n_invariants, const double* edges, int n_edges, uint32_t dims_mask,
                                          int coord_f32, double* T_channels, int ptr_kind) {
  if (!p || !u_hat || !T_channels || !invariants) {
    fit_set_error("NULL argument");
    return FIT_ERR_ARG;
  }
  if (decomposition != FIT_DECOMP_HELICAL && decomposition != FIT_DECOMP_HELMHOLTZ &&
      decomposition != FIT_DECOMP_TOROIDAL_POLOIDAL) {
    fit_set_error("calculate_partial_fluxes needs a decomposition that splits u into >=2 named components");
    return FIT_ERR_ARG;
  }
  if (p->M != p->nd || p->Dadv != p->nd) {
    fit_set_error("partial fluxes need an nd-component velocity plan");
    return FIT_ERR_ARG;
  }
  if (decomposition == FIT_DECOMP_TOROIDAL_POLOIDAL && p->nd != 3) {
    fit_set_error("ToroidalPoloidalDecomposition is defined in 3D only (got nd=%d).", p->nd);
    return FIT_ERR_ARG;
  }
  if (decomposition == FIT_DECOMP_HELICAL && p->nd != 3) {
    fit_set_error("HelicalDecomposition is defined in 3D only (got nd=%d).", p->nd);
    return FIT_ERR_ARG;
  }
  if (decomposition == FIT_DECOMP_HELMHOLTZ && p->nd != 2) {
    fit_set_error("Helmholtz decomposition currently supports 2D fields only.");
    return FIT_ERR_ARG;
  }
  if (n_invariants < 1 || n_invariants > 4) {
    fit_set_error("n_invariants must be 1..4 (got %d)", n_invariants);
    return FIT_ERR_ARG;
  }
  for (int j = 0; j < n_invariants; ++j) {
    const int inv = invariants[j];
    if (inv != INV_KE && inv != INV_HELICITY && inv != INV_ENSTROPHY) {
      fit_set_error("partial fluxes take KineticEnergy, Helicity or Enstrophy (got %d)", inv);
      return FIT_ERR_ARG;
    }
    if (inv == INV_HELICITY && p->nd != 3) {
      fit_set_error("Helicity transfer is defined in 3D only (got nd=%d).", p->nd);
      return FIT_ERR_ARG;
    }
  }
  const size_t fb = (p->io_f64 ? 16 : 8) * (size_t)p->g.Ntot * p->M;
  const void* ud = u_hat;
  if (ptr_kind != FIT_PTR_DEVICE) {
    FIT_TRY(ensure(p, &p->in_u, fb));
    FIT_CUDA_CHECK(cudaMemcpyAsync(p->in_u.p, u_hat, fb, cudaMemcpyHostToDevice, p->stream));
    ud = p->in_u.p;
  }
  FIT_TRY(ensure_shells(p, edges, n_edges, dims_mask, coord_f32));
  const size_t ob = sizeof(double) * 8 * (size_t)n_invariants * p->nsh;
  double* Td = T_channels;
  if (ptr_kind != FIT_PTR_DEVICE) {
    FIT_TRY(ensure(p, &p->outd, ob));
    Td = (double*)p->outd.p;
  }
  FIT_TRY(partial_batched(p, ud, decomposition, invariants, n_invariants, Td));
  FIT_TRY(partial_box_check(p));
  if (ptr_kind != FIT_PTR_DEVICE) {
    FIT_CUDA_CHECK(cudaMemcpyAsync(T_channels, Td, ob, cudaMemcpyDeviceToHost, p->stream));
    FIT_CUDA_CHECK(cudaStreamSynchronize(p->stream));
  }
  return FIT_OK;
}
