// Shared-memory Stockham FFT engine (radix 2/3/4/5/8, FP32 or FP64) and its pass kernels.
//
// One CTA transforms a tile of C lines at once. The tile lives in shared memory as
// [element][column] with an XOR swizzle on the column (element e of column c at
// r(e)*C + (c ^ (e & (C-1)))), so that both access shapes used here are bank-conflict free:
// lanes running along columns (strided passes, every butterfly stage) and lanes running along
// elements (the x-pass loads/stores of contiguous lines). r(e) = e, except for eight-column tiles
// of the kernels that opt in, where rows e and e ^ 1 trade places when bit 3 of e is set: with
// 8-byte elements a 16-lane phase then covers 16 different bank pairs also when its lanes span two
// rows of equal parity (the first stage's writes of rows 8j + q for two j) or eight rows apart (two
// runs of a contiguous line). With 16-byte elements (8-lane phases) and with C >= 16 the
// permutation changes no bank.
//
// Stage s of radix r, current span Ns (product of the radices before it), butterfly j:
//   inputs  x[j + q*N/r] (q < r), twiddled by w^{(j mod Ns) * q * N/(Ns*r)}, w = e^{-+2 pi i/N};
//   outputs y[q] of the radix-r DFT go to (j div Ns)*Ns*r + (j mod Ns) + q*Ns.
// This is the self-sorting (autosort) Stockham formulation: after the last stage the line is
// in natural order. All reads of a stage complete (barrier) before its writes, so one buffer
// suffices. Twiddles come from an FP64 host table (no device trigonometry).
#pragma once

#include "fit_common.cuh"

namespace fit {

// The permutation is opt-in (PERM): it pays in the 512-point strided passes and costs in the 384-
// and 256-point ones and in kernels whose registers cannot afford the second address base it needs
// in some stage shapes. A tile must be written and read with one PERM.
template <bool PERM>
FIT_D int swzp(int e, int c, int C) { return ((PERM && C == 8) ? e ^ ((e >> 3) & 1) : e) * C + (c ^ (e & (C - 1))); }
FIT_D int swz(int e, int c, int C) { return swzp<false>(e, c, C); }

// ---- radix-r DFTs in registers; INV selects e^{+2 pi i/r} --------------------------------------

template <typename V, bool INV>
FIT_D void dft2(V* v) {
  V t = v[0];
  v[0] = cadd(t, v[1]);
  v[1] = csub(t, v[1]);
}

template <typename V, bool INV>
FIT_D void dft4(V* v) {
  V t0 = cadd(v[0], v[2]), t1 = csub(v[0], v[2]);
  V t2 = cadd(v[1], v[3]), t3 = cmuli<V, INV>(csub(v[1], v[3]));
  v[0] = cadd(t0, t2);
  v[2] = csub(t0, t2);
  v[1] = cadd(t1, t3);
  v[3] = csub(t1, t3);
}

template <typename V, bool INV>
FIT_D void dft8(V* v) {
  typedef typename Scal<V>::t S;
  const S h = (S)0.70710678118654752440;
  V a[4], b[4];
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    a[q] = cadd(v[q], v[q + 4]);
    b[q] = csub(v[q], v[q + 4]);
  }
  // b[q] *= w^q, w = e^{-+2 pi i/8}
  if (!INV) {
    b[1] = mkc<V>((b[1].x + b[1].y) * h, (b[1].y - b[1].x) * h);
    b[3] = mkc<V>((b[3].y - b[3].x) * h, -(b[3].x + b[3].y) * h);
  } else {
    b[1] = mkc<V>((b[1].x - b[1].y) * h, (b[1].x + b[1].y) * h);
    b[3] = mkc<V>(-(b[3].x + b[3].y) * h, (b[3].x - b[3].y) * h);
  }
  b[2] = cmuli<V, INV>(b[2]);
  dft4<V, INV>(a);
  dft4<V, INV>(b);
  v[0] = a[0]; v[2] = a[1]; v[4] = a[2]; v[6] = a[3];
  v[1] = b[0]; v[3] = b[1]; v[5] = b[2]; v[7] = b[3];
}

template <typename V, bool INV>
FIT_D void dft3(V* v) {
  typedef typename Scal<V>::t S;
  const S s3 = (S)0.86602540378443864676;
  V t1 = cadd(v[1], v[2]);
  V t2 = csub(v[1], v[2]);
  V m = csub(v[0], cscale(t1, (S)0.5));
  V u = cscale(cmuli<V, INV>(t2), s3);
  v[0] = cadd(v[0], t1);
  v[1] = cadd(m, u);
  v[2] = csub(m, u);
}

template <typename V, bool INV>
FIT_D void dft5(V* v) {
  typedef typename Scal<V>::t S;
  const S c1 = (S)0.30901699437494742410, c2 = (S)-0.80901699437494742410;
  const S s1 = (S)0.95105651629515357212, s2 = (S)0.58778525229247312917;
  V t1 = cadd(v[1], v[4]), t2 = cadd(v[2], v[3]);
  V t3 = csub(v[1], v[4]), t4 = csub(v[2], v[3]);
  V a1 = cadd(v[0], cadd(cscale(t1, c1), cscale(t2, c2)));
  V a2 = cadd(v[0], cadd(cscale(t1, c2), cscale(t2, c1)));
  V u1 = cmuli<V, INV>(cadd(cscale(t3, s1), cscale(t4, s2)));
  V u2 = cmuli<V, INV>(csub(cscale(t3, s2), cscale(t4, s1)));
  v[0] = cadd(v[0], cadd(t1, t2));
  v[1] = cadd(a1, u1);
  v[4] = csub(a1, u1);
  v[2] = cadd(a2, u2);
  v[3] = csub(a2, u2);
}

template <typename V, int R, bool INV>
FIT_D void dftr(V* v) {
  if (R == 2) dft2<V, INV>(v);
  else if (R == 3) dft3<V, INV>(v);
  else if (R == 4) dft4<V, INV>(v);
  else if (R == 5) dft5<V, INV>(v);
  else dft8<V, INV>(v);
}

// One in-place Stockham stage over a C-column tile. EPT = tile elements per thread.
template <typename V, int R, bool INV, int EPT>
__device__ __forceinline__ void stage(V* s, int N, int C, int Ns, const V* tw, int tid, int nthr) {
  constexpr int MAXB = (EPT + R - 1) / R;
  const int NR = N / R;
  const int nb = C * NR;
  const int tstride = N / (Ns * R);
  V v[MAXB][R];
#pragma unroll
  for (int i = 0; i < MAXB; ++i) {
    const int b = tid + i * nthr;
    if (b < nb) {
      const int c = b & (C - 1);
      const int j = b / C;
      const int k = j % Ns;
#pragma unroll
      for (int q = 0; q < R; ++q) {
        V x = s[swz(j + q * NR, c, C)];
        if (q > 0 && k > 0) {
          V w = tw[k * q * tstride];
          if (INV) w.y = -w.y;
          x = cmul(x, w);
        }
        v[i][q] = x;
      }
      dftr<V, R, INV>(v[i]);
    }
  }
  __syncthreads();
#pragma unroll
  for (int i = 0; i < MAXB; ++i) {
    const int b = tid + i * nthr;
    if (b < nb) {
      const int c = b & (C - 1);
      const int j = b / C;
      const int k = j % Ns;
      const int base = (j / Ns) * Ns * R + k;
#pragma unroll
      for (int q = 0; q < R; ++q) s[swz(base + q * Ns, c, C)] = v[i][q];
    }
  }
  __syncthreads();
}

template <typename V, bool INV, int EPT>
__device__ __forceinline__ void fft_smem(V* s, int N, int C, const Radices& rd, const V* tw, int tid,
                                         int nthr) {
  int Ns = 1;
  for (int st = 0; st < rd.n; ++st) {
    const int r = rd.r[st];
    switch (r) {
      case 8: stage<V, 8, INV, EPT>(s, N, C, Ns, tw, tid, nthr); break;
      case 4: stage<V, 4, INV, EPT>(s, N, C, Ns, tw, tid, nthr); break;
      case 2: stage<V, 2, INV, EPT>(s, N, C, Ns, tw, tid, nthr); break;
      case 3: stage<V, 3, INV, EPT>(s, N, C, Ns, tw, tid, nthr); break;
      default: stage<V, 5, INV, EPT>(s, N, C, Ns, tw, tid, nthr); break;
    }
    Ns *= r;
  }
}

template <typename V>
FIT_D void load_twiddles(V* tw, const V* __restrict__ twg, int N, int tid, int nthr) {
  for (int t = tid; t < N; t += nthr) tw[t] = twg[t];
}

// ---- pass kernels ---------------------------------------------------------------------------

// Complex transform along a strided axis. Lines are indexed by (column, q): line element e of
// column col lives at  q*P*N + col + e*P  (P = product of the faster dimensions). Tiles cover C
// consecutive columns of one q. In-place use (in == out) is safe: a CTA reads its whole tile
// before writing it.
template <typename V, bool INV, int EPT>
__global__ void __launch_bounds__(1024) k_pass_strided(const V* in, V* out, int N, long P, long tilesPerQ,
                                                      int C, Radices rd, const V* __restrict__ twg,
                                                      typename Scal<V>::t scale) {
  extern __shared__ __align__(16) unsigned char fit_smem_raw[];
  V* s = reinterpret_cast<V*>(fit_smem_raw);
  V* tw = s + (size_t)C * N;
  const int tid = threadIdx.x, nthr = blockDim.x;
  const long tile = blockIdx.x;
  const long q = tile / tilesPerQ;
  const long c0 = (tile - q * tilesPerQ) * C;
  const long base = q * P * (long)N;
  const int E = C * N;
  load_twiddles(tw, twg, N, tid, nthr);
  for (int i = tid; i < E; i += nthr) {
    const int c = i & (C - 1), e = i / C;
    const long col = c0 + c;
    V x = mkc<V>(0, 0);
    if (col < P) x = in[base + col + (long)e * P];
    s[swz(e, c, C)] = x;
  }
  __syncthreads();
  fft_smem<V, INV, EPT>(s, N, C, rd, tw, tid, nthr);
  for (int i = tid; i < E; i += nthr) {
    const int c = i & (C - 1), e = i / C;
    const long col = c0 + c;
    if (col < P) out[base + col + (long)e * P] = cscale(s[swz(e, c, C)], scale);
  }
}

// Inverse real transform along x: L half-spectrum lines (N/2+1 complex, contiguous) -> L real
// lines (N, contiguous). Two real lines share one complex transform: Z = A + iB, where A, B are
// the Hermitian extensions of lines 2c and 2c+1; the imaginary parts of the self-conjugate
// bins (k = 0, k = N/2) are dropped, which is what real(ifft(.)) keeps.
template <typename V, int EPT>
__global__ void __launch_bounds__(1024) k_c2r_x(const V* __restrict__ in, typename Scal<V>::t* __restrict__ out,
                                                int N, long L, int C, Radices rd, const V* __restrict__ twg,
                                                typename Scal<V>::t scale) {
  typedef typename Scal<V>::t S;
  extern __shared__ __align__(16) unsigned char fit_smem_raw[];
  V* s = reinterpret_cast<V*>(fit_smem_raw);
  V* tw = s + (size_t)C * N;
  const int tid = threadIdx.x, nthr = blockDim.x;
  const int Nh = N / 2 + 1;
  const long l0 = (long)blockIdx.x * 2 * C;
  const int E = C * N;
  load_twiddles(tw, twg, N, tid, nthr);
  for (int i = tid; i < E; i += nthr) {
    const int c = i / N, k = i - c * N;
    const long a = l0 + 2 * c, b = a + 1;
    const bool cj = 2 * k > N;
    const int kk = cj ? N - k : k;
    const bool selfc = (k == 0) || (2 * k == N);
    V A = mkc<V>(0, 0), B = mkc<V>(0, 0);
    if (a < L) {
      A = in[a * Nh + kk];
      if (cj) A.y = -A.y;
      if (selfc) A.y = 0;
    }
    if (b < L) {
      B = in[b * Nh + kk];
      if (cj) B.y = -B.y;
      if (selfc) B.y = 0;
    }
    s[swz(k, c, C)] = mkc<V>(A.x - B.y, A.y + B.x);
  }
  __syncthreads();
  fft_smem<V, true, EPT>(s, N, C, rd, tw, tid, nthr);
  for (int i = tid; i < E; i += nthr) {
    const int c = i / N, x = i - c * N;
    const long a = l0 + 2 * c, b = a + 1;
    const V z = s[swz(x, c, C)];
    if (a < L) out[a * N + x] = z.x * scale;
    if (b < L) out[b * N + x] = z.y * scale;
  }
}

// Forward real transform along x: L real lines -> L half-spectrum lines (two-for-one packing).
template <typename V, int EPT>
__global__ void __launch_bounds__(1024) k_r2c_x(const typename Scal<V>::t* __restrict__ in, V* __restrict__ out,
                                                int N, long L, int C, Radices rd, const V* __restrict__ twg,
                                                typename Scal<V>::t scale) {
  typedef typename Scal<V>::t S;
  extern __shared__ __align__(16) unsigned char fit_smem_raw[];
  V* s = reinterpret_cast<V*>(fit_smem_raw);
  V* tw = s + (size_t)C * N;
  const int tid = threadIdx.x, nthr = blockDim.x;
  const int Nh = N / 2 + 1;
  const long l0 = (long)blockIdx.x * 2 * C;
  const int E = C * N;
  load_twiddles(tw, twg, N, tid, nthr);
  for (int i = tid; i < E; i += nthr) {
    const int c = i / N, x = i - c * N;
    const long a = l0 + 2 * c, b = a + 1;
    const S ra = (a < L) ? in[a * N + x] : (S)0;
    const S rb = (b < L) ? in[b * N + x] : (S)0;
    s[swz(x, c, C)] = mkc<V>(ra, rb);
  }
  __syncthreads();
  fft_smem<V, false, EPT>(s, N, C, rd, tw, tid, nthr);
  const S hs = (S)0.5 * scale;
  for (int i = tid; i < C * Nh; i += nthr) {
    const int c = i / Nh, k = i - c * Nh;
    const long a = l0 + 2 * c, b = a + 1;
    const V zk = s[swz(k, c, C)];
    const V zn = s[swz(k == 0 ? 0 : N - k, c, C)];
    if (a < L) out[a * Nh + k] = mkc<V>((zk.x + zn.x) * hs, (zk.y - zn.y) * hs);
    if (b < L) out[b * Nh + k] = mkc<V>((zk.y + zn.y) * hs, (zn.x - zk.x) * hs);
  }
}

}  // namespace fit

// =============================================================================================
// Compile-time engine: transform length, radix schedule, tile width and thread count are all
// template constants, so every index computation folds to shifts / constant multiplies and
// every stage is fully unrolled (no runtime radix dispatch, no local-memory spills).
// =============================================================================================
namespace fit {

__host__ __device__ constexpr int ct_p2(int n) { int p = 0; while (n % 2 == 0) { n /= 2; ++p; } return p; }
__host__ __device__ constexpr int ct_odd(int n) { while (n % 2 == 0) n /= 2; return n; }
__host__ __device__ constexpr int ct_nst(int N) {
  int p2 = ct_p2(N), n = ct_odd(N), c = p2 / 3 + (p2 % 3 != 0 ? 1 : 0);
  while (n % 3 == 0) { n /= 3; ++c; }
  while (n % 5 == 0) { n /= 5; ++c; }
  return c;
}
// Radix schedule: 8s, then 4 or 2, then 3s, then 5s; when there are two or more 8s, one 8 moves
// to the end so the first and last stages share a radix (see ct_fft_mapped).
__host__ __device__ constexpr int ct_radix_raw(int N, int s) {
  const int p2 = ct_p2(N), n8 = p2 / 3, rem = p2 % 3;
  if (s < n8) return 8;
  int idx = n8;
  if (rem) {
    if (s == idx) return rem == 2 ? 4 : 2;
    ++idx;
  }
  int n = ct_odd(N), n3 = 0;
  while (n % 3 == 0) { n /= 3; ++n3; }
  if (s < idx + n3) return 3;
  return 5;
}
__host__ __device__ constexpr int ct_radix(int N, int s) {
  const int nst = ct_nst(N), n8 = ct_p2(N) / 3;
  if (n8 >= 2 && ct_radix_raw(N, nst - 1) != 8) {
    if (s == nst - 1) return 8;
    return ct_radix_raw(N, s < n8 - 1 ? s : s + 1);
  }
  return ct_radix_raw(N, s);
}
__host__ __device__ constexpr int ct_span(int N, int s) { int p = 1; for (int i = 0; i < s; ++i) p *= ct_radix(N, i); return p; }
__host__ __device__ constexpr int ct_pow2floor(int x) { int p = 1; while (p * 2 <= x) p *= 2; return p; }

template <typename V, int N>
struct CtTile {
  static constexpr int VB = (int)sizeof(V);
  static constexpr int Cmin = 128 / VB;
  static constexpr int Cw = ct_pow2floor((VB == 8 ? 4096 : 2048) / N > 0 ? (VB == 8 ? 4096 : 2048) / N : 1);
  static constexpr int C = Cw > Cmin ? Cw : Cmin;
  static constexpr int E = C * N;
  static constexpr int EPT = E <= 8192 ? 8 : 16;
  static constexpr int NTHR = (E / EPT + 31) / 32 * 32;
  static constexpr size_t SMEM = (size_t)(E + N) * VB;
  // resident blocks per SM the register budget is sized for (2048 threads per SM)
  static constexpr int MINB = NTHR >= 768 ? 2 : (NTHR >= 512 ? 3 : 4);
};

// Tile of the stand-alone passes (x: real <-> half spectrum along contiguous lines; strided y and z):
// a 16-column tile that would need more than 512 threads is halved (block-wide barriers over fewer
// warps, several resident blocks instead of one). The x passes' staged loads and real-pair split are
// coalesced for any column count; the strided passes still read 64-byte row runs. The z pass that
// stores the full spectrum keeps 16 columns: its conjugate-mirror stores want the longer runs.
template <typename V, int N>
struct CtXTile {
  static constexpr int VB = (int)sizeof(V);
  static constexpr int C = (CtTile<V, N>::C >= 16 && CtTile<V, N>::NTHR > 512) ? CtTile<V, N>::C / 2
                                                                             : CtTile<V, N>::C;
  static constexpr int E = C * N;
  static constexpr int EPT = E <= 8192 ? 8 : 16;
  static constexpr int NTHR = (E / EPT + 31) / 32 * 32;
  static constexpr size_t SMEM = (size_t)(E + N) * VB;
};

template <typename V, bool INV, int N, int C, int NTHR, int EPT, int R, int NS, bool PERM = false>
__device__ __forceinline__ void ct_stage(V* s, const V* tw, int tid) {
  constexpr int MAXB = (EPT + R - 1) / R;
  constexpr int NR = N / R;
  constexpr int NB = C * NR;
  constexpr int TS = N / (NS * R);
  V v[MAXB][R];
#pragma unroll
  for (int i = 0; i < MAXB; ++i) {
    const int b = tid + i * NTHR;
    if (NB % NTHR == 0 || b < NB) {
      const int c = b % C;
      const int j = b / C;
      const int k = j % NS;
#pragma unroll
      for (int q = 0; q < R; ++q) {
        V x = s[swzp<PERM>(j + q * NR, c, C)];
        if (NS > 1 && q > 0) {
          V w = tw[k * q * TS];
          if (INV) w.y = -w.y;
          x = cmul(x, w);
        }
        v[i][q] = x;
      }
      dftr<V, R, INV>(v[i]);
    }
  }
  __syncthreads();
#pragma unroll
  for (int i = 0; i < MAXB; ++i) {
    const int b = tid + i * NTHR;
    if (NB % NTHR == 0 || b < NB) {
      const int c = b % C;
      const int j = b / C;
      const int k = j % NS;
      const int base = (j / NS) * NS * R + k;
#pragma unroll
      for (int q = 0; q < R; ++q) s[swzp<PERM>(base + q * NS, c, C)] = v[i][q];
    }
  }
  __syncthreads();
}

template <typename V, bool INV, int N, int C, int NTHR, int EPT, int S, bool PERM = false>
__device__ __forceinline__ void ct_stages(V* s, const V* tw, int tid) {
  if constexpr (S < ct_nst(N)) {
    ct_stage<V, INV, N, C, NTHR, EPT, ct_radix(N, S), ct_span(N, S), PERM>(s, tw, tid);
    ct_stages<V, INV, N, C, NTHR, EPT, S + 1, PERM>(s, tw, tid);
  }
}

template <typename V, bool INV, int N>
__global__ void __launch_bounds__(CtXTile<V, N>::NTHR) k_ct_strided(const V* in, V* out, long P, long tilesPerQ,
                                                                  const V* __restrict__ twg,
                                                                  typename Scal<V>::t scale) {
  typedef CtXTile<V, N> TT;
  constexpr int C = TT::C, E = TT::E;
  extern __shared__ __align__(16) unsigned char fit_smem_raw[];
  V* s = reinterpret_cast<V*>(fit_smem_raw);
  V* tw = s + E;
  const int tid = threadIdx.x;
  const long tile = blockIdx.x;
  const long q = tile / tilesPerQ;
  const long c0 = (tile - q * tilesPerQ) * C;
  const long base = q * P * (long)N;
  for (int t = tid; t < N; t += TT::NTHR) tw[t] = twg[t];
#pragma unroll 4
  for (int i = tid; i < E; i += TT::NTHR) {
    const int c = i % C, e = i / C;
    const long col = c0 + c;
    V x = mkc<V>(0, 0);
    if (col < P) x = in[base + col + (long)e * P];
    s[swz(e, c, C)] = x;
  }
  __syncthreads();
  ct_stages<V, INV, N, C, TT::NTHR, TT::EPT, 0>(s, tw, tid);
#pragma unroll 4
  for (int i = tid; i < E; i += TT::NTHR) {
    const int c = i % C, e = i / C;
    const long col = c0 + c;
    if (col < P) out[base + col + (long)e * P] = cscale(s[swz(e, c, C)], scale);
  }
}

// Forward z pass of an unpadded 3D half spectrum (columns kx + Mh0 ky of each of the nf fields,
// z stride Mh0 N1) whose store writes the full N-grid spectrum (x fastest, field slowest): mode
// (kx, ky, kz) and, for 0 < kx < N0/2, its conjugate mirror (N0 - kx, -ky, -kz), so that no separate
// scatter pass reads the half spectrum again.
template <typename V, int N>
__global__ void __launch_bounds__(CtTile<V, N>::NTHR) k_ct_z_full(const V* __restrict__ in, V* __restrict__ out,
                                                                 int N0, int Mh0, int N1, long tilesPerQ,
                                                                 const V* __restrict__ twg) {
  typedef CtTile<V, N> TT;
  constexpr int C = TT::C, E = TT::E;
  extern __shared__ __align__(16) unsigned char fit_smem_raw[];
  V* s = reinterpret_cast<V*>(fit_smem_raw);
  V* tw = s + E;
  const int tid = threadIdx.x;
  const long tile = blockIdx.x;
  const long q = tile / tilesPerQ;
  const long P = (long)Mh0 * N1;
  const long c0 = (tile - q * tilesPerQ) * C;
  const long base = q * P * (long)N;
  const long plane = (long)N0 * N1, obase = q * plane * N;
  for (int t = tid; t < N; t += TT::NTHR) tw[t] = twg[t];
#pragma unroll 4
  for (int i = tid; i < E; i += TT::NTHR) {
    const int c = i % C, e = i / C;
    const long col = c0 + c;
    V x = mkc<V>(0, 0);
    if (col < P) x = in[base + col + (long)e * P];
    s[swz(e, c, C)] = x;
  }
  __syncthreads();
  ct_stages<V, false, N, C, TT::NTHR, TT::EPT, 0>(s, tw, tid);
#pragma unroll 4
  for (int i = tid; i < E; i += TT::NTHR) {
    const int c = i % C, kz = i / C;
    const long col = c0 + c;
    if (col < P) {
      const int kx = (int)(col % Mh0), ky = (int)(col / Mh0);
      const V v = s[swz(kz, c, C)];
      out[obase + kx + (long)N0 * ky + plane * kz] = v;
      if (kx > 0 && 2 * kx < N0) {
        V m = v;
        m.y = -m.y;
        const int my = ky == 0 ? 0 : N1 - ky, mz = kz == 0 ? 0 : N - kz;
        out[obase + (N0 - kx) + (long)N0 * my + plane * mz] = m;
      }
    }
  }
}

template <typename V, int N>
__global__ void __launch_bounds__(CtXTile<V, N>::NTHR) k_ct_c2r_x(const V* __restrict__ in,
                                                                typename Scal<V>::t* __restrict__ out, long L,
                                                                const V* __restrict__ twg,
                                                                typename Scal<V>::t scale) {
  typedef CtXTile<V, N> TT;
  constexpr int C = TT::C, E = TT::E, Nh = N / 2 + 1;
  extern __shared__ __align__(16) unsigned char fit_smem_raw[];
  V* s = reinterpret_cast<V*>(fit_smem_raw);
  V* tw = s + E;
  const int tid = threadIdx.x;
  const long l0 = (long)blockIdx.x * 2 * C;
  for (int t = tid; t < N; t += TT::NTHR) tw[t] = twg[t];
#pragma unroll 4
  for (int i = tid; i < E; i += TT::NTHR) {
    const int c = i / N, k = i % N;
    const long a = l0 + 2 * c, b = a + 1;
    const bool cj = 2 * k > N;
    const int kk = cj ? N - k : k;
    const bool selfc = (k == 0) || (2 * k == N);
    V A = mkc<V>(0, 0), B = mkc<V>(0, 0);
    if (a < L) {
      A = in[a * Nh + kk];
      if (cj) A.y = -A.y;
      if (selfc) A.y = 0;
    }
    if (b < L) {
      B = in[b * Nh + kk];
      if (cj) B.y = -B.y;
      if (selfc) B.y = 0;
    }
    s[swz(k, c, C)] = mkc<V>(A.x - B.y, A.y + B.x);
  }
  __syncthreads();
  ct_stages<V, true, N, C, TT::NTHR, TT::EPT, 0>(s, tw, tid);
#pragma unroll 4
  for (int i = tid; i < E; i += TT::NTHR) {
    const int c = i / N, x = i % N;
    const long a = l0 + 2 * c, b = a + 1;
    const V z = s[swz(x, c, C)];
    if (a < L) out[a * N + x] = z.x * scale;
    if (b < L) out[b * N + x] = z.y * scale;
  }
}

template <typename V, int N>
__global__ void __launch_bounds__(CtXTile<V, N>::NTHR) k_ct_r2c_x(const typename Scal<V>::t* __restrict__ in,
                                                                V* __restrict__ out, long L,
                                                                const V* __restrict__ twg,
                                                                typename Scal<V>::t scale) {
  typedef CtXTile<V, N> TT;
  typedef typename Scal<V>::t S;
  constexpr int C = TT::C, E = TT::E, Nh = N / 2 + 1;
  extern __shared__ __align__(16) unsigned char fit_smem_raw[];
  V* s = reinterpret_cast<V*>(fit_smem_raw);
  V* tw = s + E;
  const int tid = threadIdx.x;
  const long l0 = (long)blockIdx.x * 2 * C;
  for (int t = tid; t < N; t += TT::NTHR) tw[t] = twg[t];
#pragma unroll 4
  for (int i = tid; i < E; i += TT::NTHR) {
    const int c = i / N, x = i % N;
    const long a = l0 + 2 * c, b = a + 1;
    const S ra = (a < L) ? in[a * N + x] : (S)0;
    const S rb = (b < L) ? in[b * N + x] : (S)0;
    s[swz(x, c, C)] = mkc<V>(ra, rb);
  }
  __syncthreads();
  ct_stages<V, false, N, C, TT::NTHR, TT::EPT, 0>(s, tw, tid);
  const S hs = (S)0.5 * scale;
  for (int i = tid; i < C * Nh; i += TT::NTHR) {
    const int c = i / Nh, k = i % Nh;
    const long a = l0 + 2 * c, b = a + 1;
    const V zk = s[swz(k, c, C)];
    const V zn = s[swz(k == 0 ? 0 : N - k, c, C)];
    if (a < L) out[a * Nh + k] = mkc<V>((zk.x + zn.x) * hs, (zk.y - zn.y) * hs);
    if (b < L) out[b * Nh + k] = mkc<V>((zk.y + zn.y) * hs, (zn.x - zk.x) * hs);
  }
}

template <typename V, bool INV, int N, int C, int NTHR, int EPT, int S, int SEND, bool PERM = false>
__device__ __forceinline__ void ct_stages_range(V* s, const V* tw, int tid) {
  if constexpr (S < SEND) {
    ct_stage<V, INV, N, C, NTHR, EPT, ct_radix(N, S), ct_span(N, S), PERM>(s, tw, tid);
    ct_stages_range<V, INV, N, C, NTHR, EPT, S + 1, SEND, PERM>(s, tw, tid);
  }
}

// Element map shared by a transform's inputs and outputs: butterfly b = tid + i*NTHR of the last
// stage (radix RL) owns column b % C and rows j + q*NRL, j = b / C, q < RL.
template <int N>
struct CtMap {
  static constexpr int NST = ct_nst(N);
  static constexpr int RL = ct_radix(N, NST - 1);
  static constexpr int NRL = N / RL;
  static constexpr bool DIRECT = NST >= 2 && ct_radix(N, 0) == RL;
};

// Transform of a C-column tile whose inputs come from load(i, q, row, col) and whose outputs go to
// store(i, q, row, col, value), both on the CtMap element map. When the first and last stages share
// a radix (DIRECT), stage 0 runs on the loaded registers and the last stage hands its registers to
// store, so only the inner stage exchanges touch shared memory; otherwise the map is staged through
// shared memory around the full stage sequence. store may write the element it receives back into s
// (each thread only rewrites rows it just read). Callers synchronise before reusing s.
// LOAD_S: load() reads the tile in s itself; the first stage then waits for every thread's loads
// before it overwrites s.
template <typename V, bool INV, int N, int C, int NTHR, int EPT, bool LOAD_S = false, bool PERM = false, typename LD,
          typename ST>
__device__ __forceinline__ void ct_fft_mapped(V* s, const V* tw, int tid, LD load, ST store) {
  typedef CtMap<N> MP;
  constexpr int RL = MP::RL, NRL = MP::NRL;
  constexpr int MB = (EPT + RL - 1) / RL;
  constexpr int NB = C * NRL;
  V v[MB][RL];
  if constexpr (MP::DIRECT) {
#pragma unroll
    for (int i = 0; i < MB; ++i) {
      const int b = tid + i * NTHR;
      if (NB % NTHR == 0 || b < NB) {
        const int c = b % C, j = b / C;
#pragma unroll
        for (int q = 0; q < RL; ++q) v[i][q] = load(i, q, j + q * NRL, c);
        dftr<V, RL, INV>(v[i]);
        if constexpr (!LOAD_S) {
#pragma unroll
          for (int q = 0; q < RL; ++q) s[swzp<PERM>(j * RL + q, c, C)] = v[i][q];
        }
      }
    }
    if constexpr (LOAD_S) {
      __syncthreads();
#pragma unroll
      for (int i = 0; i < MB; ++i) {
        const int b = tid + i * NTHR;
        if (NB % NTHR == 0 || b < NB) {
          const int c = b % C, j = b / C;
#pragma unroll
          for (int q = 0; q < RL; ++q) s[swzp<PERM>(j * RL + q, c, C)] = v[i][q];
        }
      }
    }
    __syncthreads();
    ct_stages_range<V, INV, N, C, NTHR, EPT, 1, MP::NST - 1, PERM>(s, tw, tid);
#pragma unroll
    for (int i = 0; i < MB; ++i) {
      const int b = tid + i * NTHR;
      if (NB % NTHR == 0 || b < NB) {
        const int c = b % C, j = b / C;
#pragma unroll
        for (int q = 0; q < RL; ++q) {
          V x = s[swzp<PERM>(j + q * NRL, c, C)];
          if (q > 0) {
            V w = tw[j * q];
            if (INV) w.y = -w.y;
            x = cmul(x, w);
          }
          v[i][q] = x;
        }
        dftr<V, RL, INV>(v[i]);
#pragma unroll
        for (int q = 0; q < RL; ++q) store(i, q, j + q * NRL, c, v[i][q]);
      }
    }
  } else {
#pragma unroll
    for (int i = 0; i < MB; ++i) {
      const int b = tid + i * NTHR;
      if (NB % NTHR == 0 || b < NB) {
        const int c = b % C, j = b / C;
#pragma unroll
        for (int q = 0; q < RL; ++q) s[swzp<PERM>(j + q * NRL, c, C)] = load(i, q, j + q * NRL, c);
      }
    }
    __syncthreads();
    ct_stages<V, INV, N, C, NTHR, EPT, 0, PERM>(s, tw, tid);
#pragma unroll
    for (int i = 0; i < MB; ++i) {
      const int b = tid + i * NTHR;
      if (NB % NTHR == 0 || b < NB) {
        const int c = b % C, j = b / C;
#pragma unroll
        for (int q = 0; q < RL; ++q) store(i, q, j + q * NRL, c, s[swzp<PERM>(j + q * NRL, c, C)]);
      }
    }
  }
}

// ct_fft_mapped with a hook between the inner stages and the last one: mid() runs on every thread
// (it may synchronise the block) and returns false to abandon the transform (then store is never
// called). Used where the last stage's consumer needs data that arrives while the transform runs.
template <typename V, bool INV, int N, int C, int NTHR, int EPT, typename LD, typename MID, typename ST>
__device__ __forceinline__ bool ct_fft_mapped_mid(V* s, const V* tw, int tid, LD load, MID mid, ST store) {
  typedef CtMap<N> MP;
  constexpr int RL = MP::RL, NRL = MP::NRL;
  constexpr int MB = (EPT + RL - 1) / RL;
  constexpr int NB = C * NRL;
  V v[MB][RL];
  if constexpr (MP::DIRECT) {
#pragma unroll
    for (int i = 0; i < MB; ++i) {
      const int b = tid + i * NTHR;
      if (NB % NTHR == 0 || b < NB) {
        const int c = b % C, j = b / C;
#pragma unroll
        for (int q = 0; q < RL; ++q) v[i][q] = load(i, q, j + q * NRL, c);
        dftr<V, RL, INV>(v[i]);
#pragma unroll
        for (int q = 0; q < RL; ++q) s[swz(j * RL + q, c, C)] = v[i][q];
      }
    }
    __syncthreads();
    ct_stages_range<V, INV, N, C, NTHR, EPT, 1, MP::NST - 1>(s, tw, tid);
    if (!mid()) return false;
#pragma unroll
    for (int i = 0; i < MB; ++i) {
      const int b = tid + i * NTHR;
      if (NB % NTHR == 0 || b < NB) {
        const int c = b % C, j = b / C;
#pragma unroll
        for (int q = 0; q < RL; ++q) {
          V x = s[swz(j + q * NRL, c, C)];
          if (q > 0) {
            V w = tw[j * q];
            if (INV) w.y = -w.y;
            x = cmul(x, w);
          }
          v[i][q] = x;
        }
        dftr<V, RL, INV>(v[i]);
#pragma unroll
        for (int q = 0; q < RL; ++q) store(i, q, j + q * NRL, c, v[i][q]);
      }
    }
  } else {
#pragma unroll
    for (int i = 0; i < MB; ++i) {
      const int b = tid + i * NTHR;
      if (NB % NTHR == 0 || b < NB) {
        const int c = b % C, j = b / C;
#pragma unroll
        for (int q = 0; q < RL; ++q) s[swz(j + q * NRL, c, C)] = load(i, q, j + q * NRL, c);
      }
    }
    __syncthreads();
    ct_stages<V, INV, N, C, NTHR, EPT, 0>(s, tw, tid);
    if (!mid()) return false;
#pragma unroll
    for (int i = 0; i < MB; ++i) {
      const int b = tid + i * NTHR;
      if (NB % NTHR == 0 || b < NB) {
        const int c = b % C, j = b / C;
#pragma unroll
        for (int q = 0; q < RL; ++q) store(i, q, j + q * NRL, c, s[swz(j + q * NRL, c, C)]);
      }
    }
  }
  return true;
}

}  // namespace fit
