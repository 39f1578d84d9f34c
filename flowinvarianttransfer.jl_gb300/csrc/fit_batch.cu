// Uneven batches: many spectral-flux instances (different grids, dimensions, invariants and shell
// geometries, one plan each) executed as ONE CUDA graph launch.
//
// The first fit_batch_run executes every instance eagerly on the caller's stream: workspaces are
// allocated and, when the autotuner is on, every transform-pass shape picks its kernel there. The
// second run captures all instances into one graph, distributed round-robin over branch streams
// (fork/join events), so small instances run side by side; every later run is one cudaGraphLaunch.
// Inputs and outputs are device pointers fixed at fit_batch_add_flux time: to process new data,
// write it into the same buffers and run again.
#include <new>
#include <vector>

#include "fit_gb300.h"
#include "fit_plan.cuh"

struct fit_batch_inst {
  fit_plan* p;
  const void* u;
  const void* a;
  int inv;
  double* T;
  double* Pi;
};

struct fit_batch {
  std::vector<fit_batch_inst> inst;
  int nbranch = 4;
  std::vector<cudaStream_t> br;
  std::vector<cudaEvent_t> join;
  cudaEvent_t fork = nullptr;
  cudaStream_t origin = nullptr;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  int state = 0;   // 0: not run, 1: eager run done, 2: graph ready
  long graph_kernels = 0;
};

namespace fit {

// Pi = +cumsum(T) over the shells (src/SpectralFlux.jl:176), one thread: n is a few hundred at most.
__global__ void k_cumsum(const double* __restrict__ T, double* __restrict__ Pi, int n) {
  if (blockIdx.x != 0 || threadIdx.x != 0) return;
  double acc = 0.0;
  for (int i = 0; i < n; ++i) {
    acc += T[i];
    Pi[i] = acc;
  }
}

template <typename T>
static int flux_device(fit_plan* p, const fit_batch_inst& in) {
  if (sizeof(T) == 4 && fz_box_ok(p)) {   // FP32 cubic 3D of a fused size: the live-box form
    FIT_TRY(s2s_box_flux(p, in.u, in.a ? in.a : in.u, in.u, in.inv, in.T));
  } else {
    FIT_TRY(nonlinear_half<T>(p, in.u, in.a, 0, false));
    FIT_TRY(carrier_and_bin_setup<T>(p, in.u, in.inv));
    FIT_TRY(bin_into<T>(p, p->nh.p, 0, 1, p->ceff.p, in.T));
  }
  if (in.Pi) {
    k_cumsum<<<1, 32, 0, p->stream>>>(in.T, in.Pi, p->nsh);
    FIT_LAUNCH_CHECK();
  }
  return FIT_OK;
}

static int run_one(const fit_batch_inst& in, cudaStream_t st) {
  cudaStream_t keep = in.p->stream;
  in.p->stream = st;
  const int rc = in.p->prec == 64 ? flux_device<double>(in.p, in) : flux_device<float>(in.p, in);
  in.p->stream = keep;
  return rc;
}

static void drop_graph(fit_batch* b) {
  if (b->exec) cudaGraphExecDestroy(b->exec);
  if (b->graph) cudaGraphDestroy(b->graph);
  b->exec = nullptr;
  b->graph = nullptr;
}

static int capture(fit_batch* b, cudaStream_t st) {
  if (!b->origin) {
    FIT_CUDA_CHECK(cudaStreamCreateWithFlags(&b->origin, cudaStreamNonBlocking));
    FIT_CUDA_CHECK(cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming));
    b->br.resize(b->nbranch);
    b->join.resize(b->nbranch);
    for (int k = 0; k < b->nbranch; ++k) {
      FIT_CUDA_CHECK(cudaStreamCreateWithFlags(&b->br[k], cudaStreamNonBlocking));
      FIT_CUDA_CHECK(cudaEventCreateWithFlags(&b->join[k], cudaEventDisableTiming));
    }
  }
  FIT_CUDA_CHECK(cudaStreamSynchronize(st));
  const long l0 = fit_launch_total();
  FIT_CUDA_CHECK(cudaStreamBeginCapture(b->origin, cudaStreamCaptureModeThreadLocal));
  int rc = FIT_OK;
  cudaError_t e = cudaEventRecord(b->fork, b->origin);
  for (int k = 0; k < b->nbranch && e == cudaSuccess; ++k) e = cudaStreamWaitEvent(b->br[k], b->fork, 0);
  if (e != cudaSuccess) {
    fit_set_error("batch capture fork failed: %s", cudaGetErrorString(e));
    rc = FIT_ERR_CUDA;
  }
  for (size_t i = 0; i < b->inst.size() && rc == FIT_OK; ++i) rc = run_one(b->inst[i], b->br[i % b->nbranch]);
  for (int k = 0; k < b->nbranch && rc == FIT_OK; ++k) {
    e = cudaEventRecord(b->join[k], b->br[k]);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(b->origin, b->join[k], 0);
    if (e != cudaSuccess) {
      fit_set_error("batch capture join failed: %s", cudaGetErrorString(e));
      rc = FIT_ERR_CUDA;
    }
  }
  cudaGraph_t g = nullptr;
  const cudaError_t ee = cudaStreamEndCapture(b->origin, &g);
  const long captured = fit_launch_total() - l0;
  fit_count_launches(-captured);   // captured launches run when the graph is launched
  if (rc != FIT_OK) {
    if (g) cudaGraphDestroy(g);
    cudaGetLastError();
    return rc;
  }
  if (ee != cudaSuccess || !g) {
    fit_set_error("batch capture failed: %s", cudaGetErrorString(ee));
    return FIT_ERR_CUDA;
  }
  b->graph = g;
  cudaError_t ie = cudaGraphInstantiate(&b->exec, g, 0);
  if (ie != cudaSuccess) {
    drop_graph(b);
    fit_set_error("batch graph instantiation failed: %s", cudaGetErrorString(ie));
    return FIT_ERR_CUDA;
  }
  size_t nn = 0;
  FIT_CUDA_CHECK(cudaGraphGetNodes(g, nullptr, &nn));
  std::vector<cudaGraphNode_t> nodes(nn);
  FIT_CUDA_CHECK(cudaGraphGetNodes(g, nodes.data(), &nn));
  long nk = 0;
  for (size_t i = 0; i < nn; ++i) {
    cudaGraphNodeType ty;
    if (cudaGraphNodeGetType(nodes[i], &ty) == cudaSuccess && ty == cudaGraphNodeTypeKernel) ++nk;
  }
  b->graph_kernels = nk;
  return FIT_OK;
}

}  // namespace fit

using namespace fit;

extern "C" {

int fit_batch_create(fit_batch** out, int n_branches) {
  if (!out) {
    fit_set_error("NULL argument");
    return FIT_ERR_ARG;
  }
  if (n_branches < 1 || n_branches > 32) {
    fit_set_error("n_branches must be in 1..32 (got %d)", n_branches);
    return FIT_ERR_ARG;
  }
  fit_batch* b = new (std::nothrow) fit_batch();
  if (!b) {
    fit_set_error("host allocation failed");
    return FIT_ERR_ALLOC;
  }
  b->nbranch = n_branches;
  *out = b;
  return FIT_OK;
}

int fit_batch_destroy(fit_batch* b) {
  if (!b) return FIT_OK;
  if (b->origin) cudaStreamSynchronize(b->origin);
  drop_graph(b);
  for (auto s : b->br) cudaStreamDestroy(s);
  for (auto e : b->join) cudaEventDestroy(e);
  if (b->fork) cudaEventDestroy(b->fork);
  if (b->origin) cudaStreamDestroy(b->origin);
  delete b;
  return FIT_OK;
}

int fit_batch_add_flux(fit_batch* b, fit_plan* p, const void* u_dev, const void* adv_dev, const double* edges,
                       int n_edges, uint32_t dims_mask, int coord_f32, int invariant, double* T_dev,
                       double* Pi_dev) {
  if (!b || !p || !u_dev || !T_dev) {
    fit_set_error("NULL argument");
    return FIT_ERR_ARG;
  }
  if (b->state != 0) {
    fit_set_error("instances can only be added before the first fit_batch_run");
    return FIT_ERR_STATE;
  }
  for (const auto& in : b->inst)
    if (in.p == p) {
      fit_set_error("every batch instance needs its own plan (this plan is already in the batch)");
      return FIT_ERR_ARG;
    }
  if (invariant < 0 || invariant > 3) {
    fit_set_error("unknown invariant %d", invariant);
    return FIT_ERR_ARG;
  }
  if (invariant == INV_HELICITY && !(p->nd == 3 && p->M == 3)) {
    fit_set_error("Helicity transfer is defined in 3D only (got nd=%d).", p->nd);
    return FIT_ERR_ARG;
  }
  if (invariant == INV_ENSTROPHY && !((p->nd == 2 || p->nd == 3) && p->M == p->nd)) {
    fit_set_error("Enstrophy transfer needs a 2D or 3D velocity plan");
    return FIT_ERR_ARG;
  }
  if (!adv_dev && p->M < p->nd) {
    fit_set_error("self-advection needs >= nd components (pass the advecting velocity)");
    return FIT_ERR_ARG;
  }
  FIT_TRY(ensure_shells(p, edges, n_edges, dims_mask, coord_f32));
  FIT_CUDA_CHECK(cudaStreamSynchronize(p->stream));
  b->inst.push_back(fit_batch_inst{p, u_dev, adv_dev ? adv_dev : u_dev, invariant, T_dev, Pi_dev});
  return FIT_OK;
}

int fit_batch_run(fit_batch* b, void* stream) {
  if (!b) {
    fit_set_error("NULL argument");
    return FIT_ERR_ARG;
  }
  if (b->inst.empty()) return FIT_OK;
  cudaStream_t st = (cudaStream_t)stream;
  if (b->state == 0) {
    for (const auto& in : b->inst) FIT_TRY(run_one(in, st));
    FIT_CUDA_CHECK(cudaStreamSynchronize(st));
    b->state = 1;
    return FIT_OK;
  }
  if (b->state == 1) {
    FIT_TRY(capture(b, st));
    b->state = 2;
  }
  FIT_CUDA_CHECK(cudaGraphLaunch(b->exec, st));
  fit_count_launches(b->graph_kernels);
  return FIT_OK;
}

int fit_batch_run_eager(fit_batch* b, void* stream) {
  if (!b) {
    fit_set_error("NULL argument");
    return FIT_ERR_ARG;
  }
  cudaStream_t st = (cudaStream_t)stream;
  for (const auto& in : b->inst) FIT_TRY(run_one(in, st));
  if (b->state == 0) {
    FIT_CUDA_CHECK(cudaStreamSynchronize(st));
    b->state = 1;
  }
  return FIT_OK;
}

int fit_batch_info(const fit_batch* b, int64_t* out, int n) {
  if (!b || !out) {
    fit_set_error("NULL argument");
    return FIT_ERR_ARG;
  }
  const int64_t v[4] = {(int64_t)b->inst.size(), b->state, b->graph_kernels, b->nbranch};
  for (int i = 0; i < n && i < 4; ++i) out[i] = v[i];
  return FIT_OK;
}

int fit_autotune_enable(int on) {
  autotune_enable(on != 0);
  return FIT_OK;
}

int fit_autotune_clear(void) {
  autotune_clear();
  return FIT_OK;
}

int fit_autotune_info(int64_t* n_entries, int64_t* n_runtime_engine, double* ms_default, double* ms_best) {
  long n = 0, c = 0;
  double d = 0.0, bst = 0.0;
  autotune_summary(&n, &c, &d, &bst);
  if (n_entries) *n_entries = n;
  if (n_runtime_engine) *n_runtime_engine = c;
  if (ms_default) *ms_default = d;
  if (ms_best) *ms_best = bst;
  return FIT_OK;
}

int fit_autotune_entry(int64_t i, int64_t* fields, double* ms) {
  if (!fields || !ms) {
    fit_set_error("NULL argument");
    return FIT_ERR_ARG;
  }
  long f[9];
  float mb = 0.f, md = 0.f;
  if (!autotune_entry((long)i, f, &mb, &md)) {
    fit_set_error("autotune entry %lld out of range", (long long)i);
    return FIT_ERR_ARG;
  }
  for (int k = 0; k < 9; ++k) fields[k] = f[k];
  ms[0] = mb;
  ms[1] = md;
  return FIT_OK;
}

}  // extern "C"
