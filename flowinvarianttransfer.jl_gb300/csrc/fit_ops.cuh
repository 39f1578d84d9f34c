// Declarations of the host launchers in fit_passes.cu / fit_ops.cu.
#pragma once

#include "fit_common.cuh"

namespace fit {

// One transform length: radix schedule + device twiddle tables w^t = e^{-2 pi i t/N} (FP64 host
// values, rounded once to FP32 for the FP32 table).
struct Axis {
  int N;
  Radices rd;
  float2* tw32;
  double2* tw64;
};

template <typename T>
const typename Vec2<T>::t* axis_tw(const Axis& a);
template <>
inline const float2* axis_tw<float>(const Axis& a) { return a.tw32; }
template <>
inline const double2* axis_tw<double>(const Axis& a) { return a.tw64; }

int axis_init(Axis* a, int N);
void axis_free(Axis* a);

// ---- transform passes (fit_passes.cu) --------------------------------------------------------
template <typename T>
int pass_strided(const typename Vec2<T>::t* in, typename Vec2<T>::t* out, const Axis& ax, long P, long Q,
                 bool inverse, T scale, cudaStream_t st);
template <typename T>
int pass_c2r_x(const typename Vec2<T>::t* in, T* out, const Axis& ax, long L, T scale, cudaStream_t st);
template <typename T>
int pass_r2c_x(const T* in, typename Vec2<T>::t* out, const Axis& ax, long L, T scale, cudaStream_t st);

// Full multi-dimensional transforms of nf contiguous fields on grid g (half spectrum <-> physical).
template <typename T>
int inverse_nd(typename Vec2<T>::t* half, T* phys, const GridDesc& g, const Axis* ax, long nf, T scale,
               cudaStream_t st);
template <typename T>
int forward_nd(const T* phys, typename Vec2<T>::t* half, const GridDesc& g, const Axis* ax, long nf, T scale,
               cudaStream_t st);
// forward_nd straight into the full N-grid spectrum (x fastest, field slowest) of unpadded 3D grids:
// the z pass stores every mode and its conjugate mirror. Returns 1 (nothing launched) when the grid
// is not an unpadded 3D grid or its z length has no compile-time kernel.
template <typename T>
int forward_nd_full(const T* phys, typename Vec2<T>::t* half, typename Vec2<T>::t* full, const GridDesc& g,
                    const Axis* ax, long nf, T scale, cudaStream_t st);

// Pass autotuner (fit_passes.cu): on/off, reset, summary and per-entry readout.
void autotune_enable(bool on);
void autotune_clear();
void autotune_summary(long* n, long* changed, double* ms_default, double* ms_best);
bool autotune_entry(long i, long* fields, float* ms_best, float* ms_default);

// ---- pointwise / reduction kernels (fit_ops.cu) ----------------------------------------------

// Wavenumber tables of the data grid (FFTW order) as device pointers: FP64, and their FP32
// roundings for the single-precision kernels (absent where a caller builds a table of its own).
struct KTab {
  const double* k[3] = {nullptr, nullptr, nullptr};
  const float* k32[3] = {nullptr, nullptr, nullptr};
};

// Wavenumber of axis d at index i in the arithmetic type CT (FP32 reads the FP32 table when present).
template <typename CT>
__device__ __forceinline__ CT ktab_at(const KTab& kt, int d, int i) {
  if constexpr (sizeof(CT) == 4) {
    if (kt.k32[d]) return kt.k32[d][i];
  }
  return (CT)kt.k[d][i];
}

// Describes one half-spectrum field to build on the transform grid: Herm(op(F)) with
//   op(F)(k) = scale * F[src][comp](k) * keep(k) * [shell(k) == band] * (i ks_d(k) if deriv >= 0).
struct GatherField {
  int src;     // 0 or 1 (two source arrays)
  int comp;    // component of the source
  int deriv;   // derivative axis or -1
  int band;    // 1-based shell restriction, 0 = none
  int filt;    // 1: multiply by the filter response G(|k|, ell) of GatherArgs
  int wband;   // 1-based smooth band: multiply by its weight from GatherArgs::wtab, 0 = none
};
struct GatherArgs {
  const void* src[2];
  long src_comp_stride[2];  // elements between components of a source (normally Ntot)
  int in_f64;               // source element type: 1 complex128, 0 complex64
  int two_thirds;
  const uint16_t* shell_full;  // N-grid shell table (needed when band > 0)
  int nfields;
  GatherField f[16];
  double scale;
  int filter_kind;   // 0 sharp, 1 Gaussian, 2 top-hat (src/Filters.jl:19-26)
  double ell;        // filter scale
  const void* wtab;  // smooth-band weights on the transform grid's half spectrum, [band][Mhalf]
  int w_f64;         // wtab element type: 1 double, 0 float
};

// Spectral filter response G(k, ell) (src/Filters.jl:19-26): sharp 1[|k| < pi/ell], Gaussian
// exp(-k^2 ell^2 / 24), top-hat sinc(k ell / (2 pi)) with the normalised sinc.
__device__ __forceinline__ double filter_response(int kind, double k, double ell) {
  const double PI = 3.14159265358979323846;
  if (kind == 0) return fabs(k) < PI / ell ? 1.0 : 0.0;
  if (kind == 1) return exp(-k * k * ell * ell / 24.0);
  const double x = k * ell / (2.0 * PI);
  if (x == 0.0) return 1.0;
  return sin(PI * x) / (PI * x);
}
template <typename T>
int gather_half(const GridDesc& g, const KTab& kt, const GatherArgs& a, typename Vec2<T>::t* out, cudaStream_t st);

// N_i = sum_j u_j * grad[i*nd + j] for i < M (physical fields, n points each).
template <typename T>
int product(const T* u, const T* grad, T* out, int nd, int M, long n, cudaStream_t st);

// Effective carrier and shell map on the transform grid's half spectrum (see fit_ops.cu).
enum Invariant { INV_KE = 0, INV_SCALAR = 1, INV_HELICITY = 2, INV_ENSTROPHY = 3 };
template <typename T>
int effective_carrier(const GridDesc& g, const KTab& kt, const void* carrier, int in_f64, long comp_stride,
                      int ncomp_carrier, int invariant, int two_thirds, const uint16_t* shell_full,
                      typename Vec2<T>::t* ceff, int nceff, uint16_t* seff, cudaStream_t st);

// Output rows of a multi-carrier binning pass: set m writes out.p[m][b*nsh + n].
struct BinOut {
  double* p[8];
};

// Shell sums of nset carrier sets against the same N̂ in one pass:
// out.p[m][b*nsh + n] = sum_{g: seff(g)=n+1} sum_c Re(conj(ceff_m,c(g)) * nh_b,c(g)).
template <typename T>
int bin_density_multi(const GridDesc& g, const typename Vec2<T>::t* nh, long nh_batch_stride, int nb,
                      const typename Vec2<T>::t* ceff, long ceff_set_stride, int nset, int nc, const uint16_t* seff,
                      int nsh, double* partial, long partial_cap, const BinOut& out, cudaStream_t st,
                      long len = -1);   // modes per field (default: the half spectrum, g.Mhalf)

// Shell sums: out[b*nsh + n] = sum_{g: seff(g)=n+1} sum_c Re(conj(ceff_c(g)) * nh_b,c(g)).
template <typename T>
int bin_density(const GridDesc& g, const typename Vec2<T>::t* nh, long nh_batch_stride, int nb,
                const typename Vec2<T>::t* ceff, int nc, const uint16_t* seff, int nsh, double* partial,
                long partial_cap, double* out, cudaStream_t st);

// Copies the box of modes every axis keeps under the 2/3 rule (indices [0, K_d] and [N_d - K_d, N_d),
// K_d = N_d/3 - 1) of ncomp column-major 3D fields from src to the same positions of dst; elements of
// eb = 8 or 16 bytes. src may be host memory the device can address (pinned, mapped): the device
// then reads it over the host link itself.
int copy_kept_box(const void* src, void* dst, const int* N, int ncomp, int eb, cudaStream_t st);
// The same copy restricted to the kept rows whose |signed y frequency| lies in [ya, yb), on at most
// max_blocks blocks of 256 threads (0: no limit).
int copy_kept_rows(const void* src, void* dst, const int* N, int ncomp, int eb, int ya, int yb, int max_blocks,
                   cudaStream_t st);

// Half spectrum on the transform grid -> full N-grid array (user layout), 2/3 mask applied.
template <typename T>
int scatter_full(const GridDesc& g, const typename Vec2<T>::t* half, int nf, int two_thirds, void* out,
                 int out_f64, cudaStream_t st);

// Shell index of every N-grid mode (1-based, 0 = none), exactly as assign_shells does.
int shell_table(const GridDesc& g, const KTab& kt, unsigned dims_mask, const double* edges, int nedges,
                int coord_f32, uint16_t* out, cudaStream_t st);
int shell_table_i64(const GridDesc& g, const uint16_t* sh, int64_t* out, cudaStream_t st);
// A caller's shell index (Int64, 1-based, 0 = none; device memory) as the uint16 table, written over
// the current one: the lowest position of an entry outside [0, nsh] goes to *bad (which must hold ~0
// beforehand) and *changed is set to 1 when any entry differs from the table it replaces.
int shell_table_from_i64(const GridDesc& g, const int64_t* idx, int nsh, uint16_t* out, unsigned long long* bad,
                         unsigned* changed, cudaStream_t st);

// Per-mode transfer density on the full N grid: t(k) = sum_c Re(conj(C_c(k)) N_c(k)).
int density_full(const GridDesc& g, const KTab& kt, const void* carrier, const void* nhat, int in_f64,
                 int ncomp, int invariant, double* out, cudaStream_t st);

// Helical (Craya-Herring) split of a 3D field on the full N grid (src/Decomposition.jl:63-98).
int helical_split(const GridDesc& g, const KTab& kt, const void* u, int in_f64, void* up, void* um,
                  cudaStream_t st,
                  bool kept_only = false);
// Toroidal / poloidal split of a 3D field (kept_only: only the 2/3-kept modes are touched).
int toroidal_split(const GridDesc& g, const KTab& kt, const void* u, int in_f64, void* tor, void* pol, cudaStream_t st,
                   bool kept_only = false);
// Rotational / divergent (spectral Leray) split of a 2D field.
int helmholtz_split(const GridDesc& g, const KTab& kt, const void* u, int in_f64, void* rot, void* div,
                    cudaStream_t st);

// Element-type conversion of user arrays (complex128 <-> complex64 etc).
int convert_complex(const void* in, int in_f64, void* out, int out_f64, long n, cudaStream_t st);

}  // namespace fit
