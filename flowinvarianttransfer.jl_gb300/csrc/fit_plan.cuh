// Plan object shared by the C-ABI translation units.
#pragma once

#include <vector>

#include "fit_ops.cuh"

struct fit_dbuf {
  void* p = nullptr;
  size_t cap = 0;
};

struct fit_plan {
  GridDesc g;
  int nd = 0;
  int M = 0;      // advected components
  int Dadv = 0;   // advecting components
  int dealias = 0;
  int prec = 64;
  int io_f64 = 1;
  fit::Axis ax[3];
  int ax_init[3] = {0, 0, 0};
  std::vector<double> ks_host[3];
  double* ks_dev[3] = {nullptr, nullptr, nullptr};
  float* ks32_dev[3] = {nullptr, nullptr, nullptr};
  fit::KTab kt;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  size_t bytes = 0;
  long buf_gen = 0;   // bumped on every (re)allocation: captured graphs key on it
  size_t h2d_total = 0;   // bytes of host inputs copied to the device by this plan's calls

  // staging copies of host inputs (user layout, io precision)
  fit_dbuf in_u, in_a, in_c, out_c, out_c2;
  // generic nonlinear-term workspace
  fit_dbuf hs, ph, nph, nh;
  fit_dbuf ceff, seff, partial, outd;
  // shell table cache
  fit_dbuf shell_full;
  fit_dbuf flag;   // small device scratch for argument checks done on the device
  std::vector<uint16_t> idx_host;   // host copy of a shell table installed from a caller's index
  fit_dbuf edges_dev;
  std::vector<double> cached_edges;
  unsigned cached_dims = 0;
  int cached_f32 = -1;   // -2: the table was installed from a caller's shell index (fit_set_shell_index)
  int nsh = 0;
  long shell_gen = 0;    // bumped whenever the shell table changes: graphs and mode lists key on it
  // batched shell-to-shell state (fit_s2s.cu)
  void* s2s = nullptr;
  // device address of a pinned host field that the batched shell-to-shell call reads into its
  // staging buffer itself (set when the call's inputs are staged, nullptr otherwise)
  const void* kept_src = nullptr;
  // batched partial-flux state (fit_partial.cu)
  void* partial_state = nullptr;
  // smooth-band weights on the transform grid's half spectrum (fit_band.cu)
  fit_dbuf wtab;
  std::vector<double> wtab_key;
};

namespace fit {
int ensure(fit_plan* p, fit_dbuf* b, size_t bytes);
int ensure_shells(fit_plan* p, const double* edges, int n_edges, unsigned dims, int coord_f32);
// wband > 0: the advected field is multiplied by smooth-band weight wband of p->wtab instead.
template <typename T>
int nonlinear_half(fit_plan* p, const void* f_dev, const void* a_dev, int band, bool reuse_u, int wband = 0);
// Effective carrier + shell map of the plan's transform grid, and shell sums of a half-spectrum
// product against it (fit_api.cu).
template <typename T>
int carrier_and_bin_setup(fit_plan* p, const void* carrier, int inv);
template <typename T>
int bin_into(fit_plan* p, const void* nh, long bstride, int nb, const void* ceff, double* out);
int s2s_batched(fit_plan* p, const void* u_dev, const void* a_dev, int invariant, double* Tdev);
int s2s_check(fit_plan* p);
// spectral flux on the live box (FP32 cubic 3D plans of a fused size; fz_box_ok)
bool fz_box_ok(const fit_plan* p);
int s2s_box_flux(fit_plan* p, const void* u_dev, const void* a_dev, const void* c_dev, int invariant, double* Tdev);
// N̂ = FFT[(u . grad) u] through the live-box passes, as the full data-grid spectrum (user layout)
int s2s_box_nonlinear_full(fit_plan* p, const void* u_dev, void* N_full);
// the live box of the fused path: modes (kx, ky' - K, kz' - K), 0 <= kx < KX, 0 <= ky', kz' < KY, P1 = KX KY
void fz_box_geom(const fit_plan* p, int* K, int* KX, int* KY, long* P1);
// smooth band-to-band T(n, m) on the live box (FP32 cubic 3D plans of a fused size); W: FP32 band
// weights in box layout [band][kz'][kx + KX ky']
int s2s_box_bands(fit_plan* p, const void* u_dev, const void* a_dev, int n_bands, int invariant, const float* W,
                  double* Tdev);
// 1 when the batched shell-to-shell path reads the inputs only on the 2/3-kept box of modes
int s2s_reads_kept_box(const fit_plan* p);
void s2s_free(fit_plan* p);
void partial_free(fit_plan* p);
int triad_m2m(fit_plan* p, const void* u_dev, const void* a_dev, int invariant, int fp64, double* S, double* net);
}  // namespace fit
