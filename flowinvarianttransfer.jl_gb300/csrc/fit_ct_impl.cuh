// Launchers of the compile-time pass kernels for the transform lengths built into the library
// (powers of two and 3 * 2^n from 8 to 1024). Included once per precision (fit_ct32.cu,
// fit_ct64.cu) so the two halves compile in parallel.
#pragma once

#include <mutex>
#include <unordered_map>

#include "fit_fft.cuh"
#include "fit_ops.cuh"

#define FIT_CT_SIZES(X) X(8) X(12) X(16) X(24) X(32) X(48) X(64) X(96) X(128) X(192) X(256) X(384) X(512) X(768) X(1024)

namespace fit {

template <typename K>
static int ct_prep(K kern, size_t smem, int nthr) {
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

template <typename V, bool INV, int N>
static int ct_strided_n(const V* in, V* out, long P, long Q, typename Scal<V>::t scale, const V* tw, cudaStream_t st) {
  typedef CtXTile<V, N> TT;
  const long tpq = (P + TT::C - 1) / TT::C;
  const long grid = tpq * Q;
  if (grid > 2147483647L) {
    fit_set_error("grid too large");
    return FIT_ERR_SIZE;
  }
  FIT_TRY(ct_prep(k_ct_strided<V, INV, N>, TT::SMEM, TT::NTHR));
  k_ct_strided<V, INV, N><<<(unsigned)grid, TT::NTHR, TT::SMEM, st>>>(in, out, P, tpq, tw, scale);
  return FIT_OK;
}

template <typename V, int N>
static int ct_z_full_n(const V* in, V* out, int N0, int Mh0, int N1, long Q, const V* tw, cudaStream_t st) {
  typedef CtTile<V, N> TT;
  const long tpq = ((long)Mh0 * N1 + TT::C - 1) / TT::C;
  const long grid = tpq * Q;
  if (grid > 2147483647L) {
    fit_set_error("grid too large");
    return FIT_ERR_SIZE;
  }
  FIT_TRY(ct_prep(k_ct_z_full<V, N>, TT::SMEM, TT::NTHR));
  k_ct_z_full<V, N><<<(unsigned)grid, TT::NTHR, TT::SMEM, st>>>(in, out, N0, Mh0, N1, tpq, tw);
  return FIT_OK;
}

template <typename V, int N>
static int ct_c2r_n(const V* in, typename Scal<V>::t* out, long L, typename Scal<V>::t scale, const V* tw,
                    cudaStream_t st) {
  typedef CtXTile<V, N> TT;
  const long grid = (L + 2L * TT::C - 1) / (2L * TT::C);
  FIT_TRY(ct_prep(k_ct_c2r_x<V, N>, TT::SMEM, TT::NTHR));
  k_ct_c2r_x<V, N><<<(unsigned)grid, TT::NTHR, TT::SMEM, st>>>(in, out, L, tw, scale);
  return FIT_OK;
}

template <typename V, int N>
static int ct_r2c_n(const typename Scal<V>::t* in, V* out, long L, typename Scal<V>::t scale, const V* tw,
                    cudaStream_t st) {
  typedef CtXTile<V, N> TT;
  const long grid = (L + 2L * TT::C - 1) / (2L * TT::C);
  FIT_TRY(ct_prep(k_ct_r2c_x<V, N>, TT::SMEM, TT::NTHR));
  k_ct_r2c_x<V, N><<<(unsigned)grid, TT::NTHR, TT::SMEM, st>>>(in, out, L, tw, scale);
  return FIT_OK;
}

// Returns 1 when N has no compile-time kernel (the caller falls back to the runtime kernel).
template <typename T>
int ct_strided(const typename Vec2<T>::t* in, typename Vec2<T>::t* out, int N, long P, long Q, bool inv, T scale,
               const typename Vec2<T>::t* tw, cudaStream_t st) {
  typedef typename Vec2<T>::t V;
#define FIT_CT_CASE(n)                                                              \
  case n:                                                                           \
    return inv ? ct_strided_n<V, true, n>(in, out, P, Q, scale, tw, st)             \
               : ct_strided_n<V, false, n>(in, out, P, Q, scale, tw, st);
  switch (N) {
    FIT_CT_SIZES(FIT_CT_CASE)
    default: return 1;
  }
#undef FIT_CT_CASE
}

// Returns 1 when the z length has no compile-time kernel.
template <typename T>
int ct_z_full(const typename Vec2<T>::t* in, typename Vec2<T>::t* out, int N0, int Mh0, int N1, int N2, long Q,
              const typename Vec2<T>::t* tw, cudaStream_t st) {
  typedef typename Vec2<T>::t V;
#define FIT_CT_CASE(n) \
  case n: return ct_z_full_n<V, n>(in, out, N0, Mh0, N1, Q, tw, st);
  switch (N2) {
    FIT_CT_SIZES(FIT_CT_CASE)
    default: return 1;
  }
#undef FIT_CT_CASE
}

template <typename T>
int ct_c2r(const typename Vec2<T>::t* in, T* out, int N, long L, T scale, const typename Vec2<T>::t* tw,
           cudaStream_t st) {
  typedef typename Vec2<T>::t V;
#define FIT_CT_CASE(n) \
  case n: return ct_c2r_n<V, n>(in, out, L, scale, tw, st);
  switch (N) {
    FIT_CT_SIZES(FIT_CT_CASE)
    default: return 1;
  }
#undef FIT_CT_CASE
}

template <typename T>
int ct_r2c(const T* in, typename Vec2<T>::t* out, int N, long L, T scale, const typename Vec2<T>::t* tw,
           cudaStream_t st) {
  typedef typename Vec2<T>::t V;
#define FIT_CT_CASE(n) \
  case n: return ct_r2c_n<V, n>(in, out, L, scale, tw, st);
  switch (N) {
    FIT_CT_SIZES(FIT_CT_CASE)
    default: return 1;
  }
#undef FIT_CT_CASE
}

}  // namespace fit
