// Fused FP32 shell-to-shell pipeline for cubic 3D grids (2/3 or 3/2 dealiasing).
//
// Every mediator m needs N_m = (u . grad) u_m, u_m = u restricted to shell m, and then
// T(n, m) = sum over shell n of Re(conj(C) N_m). Only the "live box" of the spectrum can be
// non-zero: |k_d| <= K with K = N div 3 - 1 (2/3 rule) or K = floor(N/2) (data grid embedded in
// the 3/2 padded grid). The pipeline keeps every spectral intermediate restricted to that box
// (kx in [0, K], ky/kz in [-K, K], stored compactly with index f + K), fuses the derivative
// multipliers, masks and scalings into the transform passes, computes the physical-space
// product inside the x pass (inverse x transform -> product with the advecting velocity ->
// forward x transform in one kernel), and bins the transfer density inside the last forward
// pass (no N_m field is written):
//
//   zinv  : z pass of H * [shell == m] and of ik_z * H * [shell == m]        (6 outputs / m)
//   yinv  : y pass -> Y(ik_x P), Y(ik_y P), Y(Q)   (P, Q = the two zinv outputs) (9 outputs / m)
//   xmix  : per component c: sum_j u_j * C2R(G_cj) -> R2C -> kx <= K           (3 outputs / m)
//   yfwd  : y pass forward, keep ky in [-K, K]                                 (3 outputs / m)
//   zfwd  : z pass forward, t = sum_c Re(conj(Ceff_c) N_c), FP64 shell bins per block
//
// Layouts (complex64 unless noted): live pencils col = kx + KX*ky' (P1 = KX*KY of them);
//   H, Ceff   [c][kz'][col]           seff, sb (uint16) [kz'][col]
//   zoff/zent: the modes with sb == m of each C-pencil tile, listed per (m, tile)
//   zinv out  [b][c][v][z][col]        yinv out [b][c][j][z][y][kx]
//   xmix out  [b][c][line = y + N z][kx]   yfwd out [b][c][z][ky'][kx]
#pragma once

#include <stdlib.h>

#include <mutex>
#include <type_traits>
#include <unordered_map>

#include "fit_fft.cuh"
#include "fit_maps.cuh"
#include "fit_tma.cuh"

namespace fit {

struct FzArgs {
  int K, KX, KY;
  long P1;      // KX * KY live pencils
  long L;       // N * N lines of the x pass
  // padded row strides of the batch intermediates (multiples of 4 elements, so that every row and
  // every 8-element tile row segment starts on a 32-byte sector): KXS for the [..][line][kx] arrays
  // (y-inverse output = x-pass input, x-pass output = y-forward input), P1S for the [..][z][pencil]
  // arrays (z-inverse output = y-inverse input, y-forward output = z-forward input)
  int KXS;
  long P1S;
  int nsh;
  int nb;       // mediators in this launch
  int med[16];  // their shell numbers (1-based)
  short ext[16][3];   // per mediator: largest |signed frequency| of its shell's modes along x, y, z
  float so;     // output normalisation of the forward transform (1/Ntot, or Mtot/Ntot^2 padded)
  int xpair;    // x pass: complex column c carries lines (2c, 2c+1) (0) or (c, c+C) (1) of its tile
  // z pass inputs as lists: the modes of band shell m in pencil tile t (C consecutive pencils) are
  // zent[zoff[(m-1)*ntile + t] .. zoff[(m-1)*ntile + t + 1]), each (kz' << 6) | (pencil - t*C)
  const unsigned* zoff;
  const uint16_t* zent;
  int ntile;
  // batches of whole-box terms (partial fluxes): mediator b advects field hidx[b] of the H array
  // (3 KY P1 complex values each) by velocity uidx[b] of the U array (3 N^3 floats each)
  int hidx[16];
  int uidx[16];
  // smooth bands: when wbox is set, the z pass multiplies field hidx[b] by the weights of band
  // widx[b] (box layout [band][kz'][col], KY P1 floats per band) as it loads it
  const float* wbox;
  int widx[16];
  long long wlim;   // first bound of the x pass's copy waits (fit_wait_cycles)
  int tz0;          // zinv: first pencil tile of the launch (launches over a range of tiles)
  int nozinv;       // fz_batch: the batch's zinv outputs are already written (tile-range launches)
};

// the padded row strides of a batch's intermediates, from its KX and P1
inline void fz_set_strides(FzArgs* a) {
  a->KXS = (a->KX + 3) & ~3;
  a->P1S = (a->P1 + 3) & ~3L;
}

FIT_D int fz_freq(int e, int N) { return (2 * e <= N) ? e : e - N; }
FIT_D float2 fz_muli(float2 h, float k) { return make_float2(-h.y * k, h.x * k); }   // i*k*h

// Tile of the fused strided passes (zinv, yinv, yfwd, zfwd_bin): C pencils of N points, EPT
// elements per thread; MINB resident blocks per SM bound the registers.
template <int N>
struct FzTile {
  static constexpr int C = (N == 512 || N == 384) ? 8 : CtTile<float2, N>::C;
  static constexpr int E = C * N;
  static constexpr int EPT = E <= 8192 ? 8 : 16;
  static constexpr int NTHR = (E / EPT + 31) / 32 * 32;
  static constexpr size_t SMEM = (size_t)(E + N) * 8;
  static constexpr int MINB = (N == 512 || N == 384) ? 4 : CtTile<float2, N>::MINB;
  static constexpr int MINB_Y = MINB;     // yinv
  static constexpr int MINB_BIN = MINB;   // zfwd_bin (per-thread transfer sums stay live across transforms)
};

// ---- zinv --------------------------------------------------------------------------------------
// One block per (mediator, component and derivative, pencil tile): the tile's modes of the
// mediator's shell are scattered from their list into a zeroed tile, then transformed along z.
template <int N>
__global__ void __launch_bounds__(FzTile<N>::NTHR, FzTile<N>::MINB) k_fz_zinv(FzArgs a, const float2* __restrict__ H,
                                                                    const float* __restrict__ kd,
                                                                    float2* __restrict__ out,
                                                                    const float2* __restrict__ twg) {
  typedef FzTile<N> TT;
  constexpr bool PM = N == 512;   // permuted tile rows (see swzp) at 512 points
  constexpr int C = TT::C, E = TT::E, NT = TT::NTHR, EPT = TT::EPT;
  static_assert(C <= 64 && NT * EPT == E, "zinv: tile column must fit the list entry");
  extern __shared__ __align__(16) unsigned char fit_smem_raw[];
  float2* s = reinterpret_cast<float2*>(fit_smem_raw);
  float2* tw = s + E;
  const int tid = threadIdx.x;
  const int tile = blockIdx.z + a.tz0;
  const long c0 = (long)tile * C;
  const int c = blockIdx.y >> 1, v = blockIdx.y & 1, b = blockIdx.x;
  const int m = a.med[b];
  const int ex = a.ext[b][0], ey = a.ext[b][1];
  // pencils (kx, ky) outside the mediator's extent hold no mode of its shell: skip the tile (its
  // outputs are never read: yinv and xmix mask with the same extents)
  bool live = false;
  for (int cc = 0; cc < C && !live; ++cc) {
    const long col = c0 + cc;
    if (col >= a.P1) break;
    const int kx = (int)(col % a.KX), ky = (int)(col / a.KX) - a.K;
    live = kx <= ex && ky >= -ey && ky <= ey;
  }
  if (!live) return;
  const long tl = (long)(m - 1) * a.ntile + tile;
  const unsigned e0 = a.zoff[tl], e1 = a.zoff[tl + 1];
  float2* ob = out + (((long)b * 3 + c) * 2 + v) * N * a.P1S;
  if (e0 == e1) {   // no mode of the shell in these pencils: the transform is zero
    for (int i = tid; i < E; i += NT) {
      const int cc = i % C, e = i / C;
      if (c0 + cc < a.P1) ob[(long)e * a.P1S + c0 + cc] = make_float2(0.f, 0.f);
    }
    return;
  }
#pragma unroll
  for (int r = 0; r < EPT; ++r) s[tid + r * NT] = make_float2(0.f, 0.f);
  for (int t = tid; t < N; t += NT) tw[t] = twg[t];
  __syncthreads();
  const float2* Hc = H + (long)c * a.KY * a.P1 + c0;
  for (unsigned t = e0 + tid; t < e1; t += NT) {
    const unsigned en = a.zent[t];
    const int kz = (int)(en >> 6), cc = (int)(en & 63u);
    float2 val = Hc[(long)kz * a.P1 + cc];
    if (v) val = fz_muli(val, kd[kz]);
    const int f = kz - a.K;
    s[swzp<PM>(f < 0 ? f + N : f, cc, C)] = val;
  }
  __syncthreads();
  ct_fft_mapped<float2, true, N, C, NT, EPT, true, PM>(
      s, tw, tid, [&](int, int, int e, int cc) -> float2 { return s[swzp<PM>(e, cc, C)]; },
      [&](int, int, int e, int cc, float2 val) {
        const long col = c0 + cc;
        if (col < a.P1) ob[(long)e * a.P1S + col] = val;
      });
}

// ---- yinv --------------------------------------------------------------------------------------
template <int N>
__global__ void __launch_bounds__(FzTile<N>::NTHR, FzTile<N>::MINB_Y) k_fz_yinv(FzArgs a, const float2* __restrict__ in,
                                                                    const float* __restrict__ kd,
                                                                    float2* __restrict__ out,
                                                                    const float2* __restrict__ twg) {
  typedef FzTile<N> TT;
  constexpr bool PM = N == 512;   // permuted tile rows (see swzp) at 512 points
  constexpr int C = TT::C, E = TT::E, NT = TT::NTHR;
  extern __shared__ __align__(16) unsigned char fit_smem_raw[];
  float2* s = reinterpret_cast<float2*>(fit_smem_raw);
  float2* tw = s + E;
  const int tid = threadIdx.x;
  const int nkt = (a.KX + C - 1) / C;
  const int z = blockIdx.z / nkt, k0 = (blockIdx.z % nkt) * C;
  const int c = blockIdx.y / 3, j = blockIdx.y % 3, b = blockIdx.x;
  const int v = (j == 2) ? 1 : 0;
  const int ex = a.ext[b][0], ey = a.ext[b][1];
  if (k0 > ex) return;   // no mode of the mediator's shell at these kx (outputs never read)
  const long ib = ((((long)b * 3 + c) * 2 + v) * N + z) * a.P1S;
  // the twiddle table is first read after the transform's first stage, behind its block barrier
  for (int t = tid; t < N; t += NT) tw[t] = twg[t];
  const long obase = ((((long)b * 3 + c) * 3 + j) * N + z) * N;
  ct_fft_mapped<float2, true, N, C, NT, TT::EPT, false, PM>(
      s, tw, tid,
      [&](int, int, int e, int cc) -> float2 {
        const int kx = k0 + cc;
        const int f = fz_freq(e, N);
        float2 val = make_float2(0.f, 0.f);
        if (kx <= ex && f >= -ey && f <= ey) {
          const int ky = f + a.K;
          val = in[ib + kx + (long)a.KX * ky];
          if (j == 1) val = fz_muli(val, kd[ky]);
          if (j == 0) val = fz_muli(val, kd[a.K + kx]);   // x derivative of the j = 0 output
        }
        return val;
      },
      [&](int, int, int e, int cc, float2 val) {
        const int kx = k0 + cc;
        if (kx < a.KX) out[(obase + e) * a.KXS + kx] = val;
      });
}

// The y-inverse pass of a batch over z planes [0, nz), one block per (mediator, output, plane, kx tile).
template <int N>
int fz_yinv(const FzArgs& a, const float2* in, const float* kd, float2* out, const float2* tw, int* err, int nz,
            cudaStream_t st) {
  typedef FzTile<N> TT;
  (void)err;
  FIT_TRY(ct_prep_fused(k_fz_yinv<N>, TT::SMEM, TT::NTHR));
  const unsigned nkt = (unsigned)((a.KX + TT::C - 1) / TT::C);
  k_fz_yinv<N><<<dim3(a.nb, 9, nkt * (unsigned)nz), TT::NTHR, TT::SMEM, st>>>(a, in, kd, out, tw);
  FIT_LAUNCH_CHECK();
  return FIT_OK;
}

// ---- xmix: inverse x transforms, product with the advecting velocity, forward x transform -----
template <int N>
__global__ void __launch_bounds__(FzTile<N>::NTHR) k_fz_xmix(FzArgs a, const float2* __restrict__ G,
                                                                    const float* __restrict__ U,
                                                                    float2* __restrict__ out,
                                                                    const float2* __restrict__ twg) {
  typedef FzTile<N> TT;
  constexpr int C = TT::C, E = TT::E, NT = TT::NTHR, EPT = TT::EPT;
  static_assert(NT * EPT == E, "xmix needs an exact thread/element split");
  extern __shared__ __align__(16) unsigned char fit_smem_raw[];
  float2* s = reinterpret_cast<float2*>(fit_smem_raw);
  float2* tw = s + E;
  const int tid = threadIdx.x;
  const long l0 = (long)blockIdx.z * 2 * C;
  const int b = blockIdx.x;
  const int ex = a.ext[b][0];   // gradient inputs are zero beyond the mediator's x extent
  const long Mtot = (long)N * N * N;
  U += (long)a.uidx[b] * 3 * Mtot;   // this mediator's advecting velocity
  for (int t = tid; t < N; t += NT) tw[t] = twg[t];
  for (int c = 0; c < 3; ++c) {
    float2 acc[EPT];
#pragma unroll
    for (int r = 0; r < EPT; ++r) acc[r] = make_float2(0.f, 0.f);
    for (int j = 0; j < 3; ++j) {
      const long gb = (((long)b * 3 + c) * 3 + j) * a.L;
      __syncthreads();
#pragma unroll 4
      for (int r = 0; r < EPT; ++r) {
        const int i = tid + r * NT;
        const int col = i / N, k = i % N;
        const long la = l0 + 2 * col, lb = la + 1;
        const bool cj = 2 * k > N;
        const int kk = cj ? N - k : k;
        float2 A = make_float2(0.f, 0.f), B = make_float2(0.f, 0.f);
        if (kk <= ex) {
          if (la < a.L) A = G[(gb + la) * a.KXS + kk];
          if (lb < a.L) B = G[(gb + lb) * a.KXS + kk];
          if (cj) { A.y = -A.y; B.y = -B.y; }
          if (k == 0) { A.y = 0.f; B.y = 0.f; }
        }
        s[swz(k, col, C)] = make_float2(A.x - B.y, A.y + B.x);
      }
      __syncthreads();
      ct_stages<float2, true, N, C, NT, EPT, 0>(s, tw, tid);
      const float* Uj = U + (long)j * Mtot;
#pragma unroll 4
      for (int r = 0; r < EPT; ++r) {
        const int i = tid + r * NT;
        const int col = i / N, x = i % N;
        const long la = l0 + 2 * col, lb = la + 1;
        const float2 zv = s[swz(x, col, C)];
        const float ua = (la < a.L) ? Uj[la * N + x] : 0.f;
        const float ub = (lb < a.L) ? Uj[lb * N + x] : 0.f;
        acc[r].x += ua * zv.x;
        acc[r].y += ub * zv.y;
      }
    }
    __syncthreads();
#pragma unroll
    for (int r = 0; r < EPT; ++r) {
      const int i = tid + r * NT;
      const int col = i / N, x = i % N;
      s[swz(x, col, C)] = acc[r];
    }
    __syncthreads();
    ct_stages<float2, false, N, C, NT, EPT, 0>(s, tw, tid);
    const long obase = ((long)b * 3 + c) * a.L;
    const float hs = 0.5f * a.so;
    for (int i = tid; i < C * a.KX; i += NT) {
      const int col = i / a.KX, k = i % a.KX;
      const long la = l0 + 2 * col, lb = la + 1;
      const float2 zk = s[swz(k, col, C)];
      const float2 zn = s[swz(k == 0 ? 0 : N - k, col, C)];
      if (la < a.L) out[(obase + la) * a.KXS + k] = make_float2((zk.x + zn.x) * hs, (zk.y - zn.y) * hs);
      if (lb < a.L) out[(obase + lb) * a.KXS + k] = make_float2((zk.y + zn.y) * hs, (zn.x - zk.x) * hs);
    }
  }
}

// ---- xmix with bulk-copy staging ------------------------------------------------------------------
// Same arithmetic as k_fz_xmix. The nine gradient tiles a block consumes ((c, j) pairs; each tile is
// 2C consecutive lines x KX complex, one contiguous block of G) are streamed into two shared
// staging buffers by bulk asynchronous copies: tile t+1 is in flight while tile t is transformed.
// The advecting-velocity values a thread multiplies are loaded into registers before each inverse
// transform, so their latency overlaps the transform. C = 8 columns keeps registers below the
// two-blocks-per-SM limit.
template <int N>
struct XTile {
  static constexpr int Cw = ct_pow2floor(2048 / N > 0 ? 2048 / N : 1);
  static constexpr int C = Cw > 8 ? Cw : 8;
  static constexpr int E = C * N;
  static constexpr int EPT = E <= 8192 ? 8 : 16;
  static constexpr int NTHR = E / EPT;
  static constexpr size_t SMEM_FIXED = (((size_t)(E + N) * 8 + 16) + 127) / 128 * 128;
};

template <int N>
__global__ void __launch_bounds__(XTile<N>::NTHR, 2) k_fz_xmix_bulk(FzArgs a, const float2* __restrict__ G,
                                                                const float* __restrict__ U,
                                                                float2* __restrict__ out,
                                                                const float2* __restrict__ twg, int* err) {
  typedef XTile<N> TT;
  constexpr int C = TT::C, E = TT::E, NT = TT::NTHR, EPT = TT::EPT;
  static_assert(NT * EPT == E, "xmix needs an exact thread/element split");
  extern __shared__ __align__(128) unsigned char fit_smem_raw[];
  float2* s = reinterpret_cast<float2*>(fit_smem_raw);
  float2* tw = s + E;
  uint64_t* bar = reinterpret_cast<uint64_t*>(tw + N);
  float2* stg = reinterpret_cast<float2*>(fit_smem_raw + TT::SMEM_FIXED);
  const int SB = 2 * C * a.KXS;
  const uint32_t bytes = (uint32_t)SB * 8u;
  const int tid = threadIdx.x;
  const long l0 = (long)blockIdx.z * 2 * C;
  const int b = blockIdx.x;
  const int ex = a.ext[b][0];   // gradient inputs are zero beyond the mediator's x extent
  const long Mtot = (long)N * N * N;
  U += (long)a.uidx[b] * 3 * Mtot;   // this mediator's advecting velocity
  if (tid == 0) {
    mbar_init(&bar[0], 1);
    mbar_init(&bar[1], 1);
    mbar_init_fence();
  }
  for (int t = tid; t < N; t += NT) tw[t] = twg[t];
  __syncthreads();
  if (tid == 0) {
    const long gb = ((long)b * 3 * 3) * a.L;
    mbar_expect_tx(&bar[0], bytes);
    bulk_g2s(stg, G + (gb + l0) * a.KXS, bytes, &bar[0]);
  }
  float2 acc[EPT];
  bool failed = false;   // a first wait ran out (the second, full-bound wait then succeeded)
  for (int t = 0; t < 9; ++t) {
    const int c = t / 3, j = t % 3, buf = t & 1;
    if (j == 0) {
#pragma unroll
      for (int r = 0; r < EPT; ++r) acc[r] = make_float2(0.f, 0.f);
    }
    if (tid == 0 && t + 1 < 9) {
      const int c1 = (t + 1) / 3, j1 = (t + 1) % 3, nb1 = (t + 1) & 1;
      const long gb = (((long)b * 3 + c1) * 3 + j1) * a.L;
      fence_proxy_async_smem();
      mbar_expect_tx(&bar[nb1], bytes);
      bulk_g2s(stg + nb1 * SB, G + (gb + l0) * a.KXS, bytes, &bar[nb1]);
    }
    // advecting velocity at this thread's accumulate positions (lanes along x: coalesced), loaded
    // ahead of the transform so the loads overlap it
    const float* Uj = U + (long)j * Mtot;
    float ua[EPT], ub[EPT];
#pragma unroll
    for (int r = 0; r < EPT; ++r) {
      const int i = tid + r * NT;
      const int col = i / N, x = i % N;
      const long la = l0 + 2 * col;
      ua[r] = Uj[la * N + x];
      ub[r] = Uj[(la + 1) * N + x];
    }
    const bool ok = mbar_wait_or_flag(&bar[buf], (uint32_t)((t >> 1) & 1), a.wlim, failed);
    if (__syncthreads_or(!ok)) {
      if (tid == 0) {
        atomicExch(err, 1);
        // bounded chance for this tile and the prefetched next one to land before the block exits
        mbar_wait_bounded(&bar[buf], (uint32_t)((t >> 1) & 1), 200000000LL);
        if (t + 1 < 9) mbar_wait_bounded(&bar[(t + 1) & 1], (uint32_t)(((t + 1) >> 1) & 1), 200000000LL);
      }
      return;
    }
    const float2* sg = stg + buf * SB;
    ct_fft_mapped<float2, true, N, C, NT, EPT>(
        s, tw, tid,
        [&](int, int, int k, int col) -> float2 {
          const bool cj = 2 * k > N;
          const int kk = cj ? N - k : k;
          float2 A = make_float2(0.f, 0.f), B = make_float2(0.f, 0.f);
          if (kk <= ex) {
            A = sg[(2 * col) * a.KXS + kk];
            B = sg[(2 * col + 1) * a.KXS + kk];
            if (cj) { A.y = -A.y; B.y = -B.y; }
            if (k == 0) { A.y = 0.f; B.y = 0.f; }
          }
          return make_float2(A.x - B.y, A.y + B.x);
        },
        [&](int, int, int x, int col, float2 zv) { s[swz(x, col, C)] = zv; });
    __syncthreads();
#pragma unroll
    for (int r = 0; r < EPT; ++r) {
      const int i = tid + r * NT;
      const int col = i / N, x = i % N;
      const float2 zv = s[swz(x, col, C)];
      acc[r].x += ua[r] * zv.x;
      acc[r].y += ub[r] * zv.y;
    }
    __syncthreads();
    if (j == 2) {
#pragma unroll
      for (int r = 0; r < EPT; ++r) {
        const int i = tid + r * NT;
        const int col = i / N, x = i % N;
        s[swz(x, col, C)] = acc[r];
      }
      __syncthreads();
      ct_stages<float2, false, N, C, NT, EPT, 0>(s, tw, tid);
      const long obase = ((long)b * 3 + c) * a.L;
      const float hs = 0.5f * a.so;
      for (int i = tid; i < C * a.KX; i += NT) {
        const int col = i / a.KX, k = i % a.KX;
        const long la = l0 + 2 * col, lb = la + 1;
        const float2 zk = s[swz(k, col, C)];
        const float2 zn = s[swz(k == 0 ? 0 : N - k, col, C)];
        out[(obase + la) * a.KXS + k] = make_float2((zk.x + zn.x) * hs, (zk.y - zn.y) * hs);
        out[(obase + lb) * a.KXS + k] = make_float2((zk.y + zn.y) * hs, (zn.x - zk.x) * hs);
      }
      __syncthreads();
    }
  }
  if (failed) atomicExch(err, 1);
}

// ---- xmix, register-accumulating form -------------------------------------------------------------
// Same arithmetic as k_fz_xmix_bulk, restructured so that no transform output makes an extra round
// trip through shared memory: the advecting-velocity tile of the current j (2C lines x N floats,
// contiguous in U) is bulk-copied into shared memory, the inverse transform's last stage hands its
// outputs (butterfly order) to a store that accumulates u_j * value straight into registers, and
// the forward transform's first stage reads those registers (the element map of a transform's last
// stage is the map of the next transform's first stage). Gradient tiles are double-buffered as in
// k_fz_xmix_bulk; the single velocity buffer is refilled after each step's final barrier and waited
// for only before the last stage of the next inverse transform, so its copy overlaps two stages.
template <int N>
struct XRTile {
  static constexpr int C = XTile<N>::C;
  static constexpr int E = C * N;
  static constexpr int EPT = XTile<N>::EPT;
  static constexpr int NTHR = XTile<N>::NTHR;
  // velocity tile rows padded to N + 4 floats (16-byte aligned rows): the butterfly-order reads of
  // the 8 columns of a warp then fall on distinct banks in pairs instead of all on one bank
  static constexpr int UP = N + 4;
  static constexpr size_t U_BYTES = (size_t)2 * C * UP * 4;
  // s, twiddles, 3 mbarriers, then the velocity tile, then two gradient staging buffers
  static constexpr size_t OFF_U = (((size_t)(E + N) * 8 + 32) + 127) / 128 * 128;
  static constexpr size_t OFF_G = OFF_U + U_BYTES;
  // the register accumulators need the last stage's radix to divide the elements per thread
  static constexpr bool OK = EPT % CtMap<N>::RL == 0 && NTHR * EPT == E;
};

template <int N>
__global__ void __launch_bounds__(XRTile<N>::NTHR, 2) k_fz_xmix_reg(FzArgs a, const float2* __restrict__ G,
                                                                const float* __restrict__ U,
                                                                float2* __restrict__ out,
                                                                const float2* __restrict__ twg, int* err) {
  typedef XRTile<N> TT;
  constexpr int C = TT::C, NT = TT::NTHR, EPT = TT::EPT;
  typedef CtMap<N> MP;
  constexpr int RL = MP::RL;
  constexpr int MB = (EPT + RL - 1) / RL;
  static_assert(MB * RL == EPT && NT * EPT == TT::E, "xmix needs an exact thread/element split");
  extern __shared__ __align__(128) unsigned char fit_smem_raw[];
  float2* s = reinterpret_cast<float2*>(fit_smem_raw);
  float2* tw = s + TT::E;
  uint64_t* bar = reinterpret_cast<uint64_t*>(tw + N);   // [0],[1] gradient buffers, [2] velocity
  float* us = reinterpret_cast<float*>(fit_smem_raw + TT::OFF_U);
  float2* stg = reinterpret_cast<float2*>(fit_smem_raw + TT::OFF_G);
  const int SB = 2 * C * a.KXS;
  const uint32_t gbytes = (uint32_t)SB * 8u;
  const int tid = threadIdx.x;
  const long l0 = (long)blockIdx.z * 2 * C;
  const int b = blockIdx.x;
  const int ex = a.ext[b][0];   // gradient inputs are zero beyond the mediator's x extent
  const long Mtot = (long)N * N * N;
  U += (long)a.uidx[b] * 3 * Mtot;   // this mediator's advecting velocity
  // the two lines of complex column c: gradient rows ra, rb of the (line-ordered) staging tile;
  // velocity line r lands in row urow(r), so that column c reads velocity rows c and c + C
  // (4-bank row offsets with rows of N + 4 floats: conflict-free for a warp's 8 columns)
  const int xp = a.xpair;
  auto urow = [&](int r) -> int { return xp ? r : (r & 1) * C + (r >> 1); };
  if (tid == 0) {
    mbar_init(&bar[0], 1);
    mbar_init(&bar[1], 1);
    mbar_init(&bar[2], 1);
    mbar_init_fence();
  }
  for (int t = tid; t < N; t += NT) tw[t] = twg[t];
  __syncthreads();
  if (tid == 0) {
    const long gb = ((long)b * 3 * 3) * a.L;
    mbar_expect_tx(&bar[0], gbytes);
    bulk_g2s(stg, G + (gb + l0) * a.KXS, gbytes, &bar[0]);
    mbar_expect_tx(&bar[2], (uint32_t)(2 * C * N * 4));
    for (int r = 0; r < 2 * C; ++r) bulk_g2s(us + urow(r) * TT::UP, U + (l0 + r) * N, (uint32_t)(N * 4), &bar[2]);
  }
  // Every thread waits on the copy barriers itself (the completed phase makes the bulk-copied data
  // visible to it), so no block barrier is spent on the waits. A first wait that runs out marks
  // the launch failed (the flag tells the host to discard the result) and is followed by a second
  // wait with the full bound, which keeps the barrier phases in step with the issued copies. When
  // that one runs out as well the thread is "broken": the block carries on with whatever the tile
  // holds (indices never depend on data, so every access stays in bounds and every thread reaches
  // the same barriers). Thread 0 waits on every phase too and stops issuing copies once it is
  // broken, so every later wait is bounded as well; it counts the phases it issued per barrier
  // and, before the block exits, waits for the last one of each, so no copy is still landing.
  bool failed = false, broken = false;
  int issued0 = 1, issued1 = 0, issued2 = 1;   // phases issued on bars 0, 1, 2 (thread 0)
  float2 acc[MB][RL];
  for (int t = 0; t < 9; ++t) {
    const int c = t / 3, j = t % 3, buf = t & 1;
    if (j == 0) {
#pragma unroll
      for (int i = 0; i < MB; ++i)
#pragma unroll
        for (int q = 0; q < RL; ++q) acc[i][q] = make_float2(0.f, 0.f);
    }
    if (tid == 0 && t + 1 < 9 && !broken) {   // once broken, issue nothing more
      const int c1 = (t + 1) / 3, j1 = (t + 1) % 3, nb1 = (t + 1) & 1;
      const long gb = (((long)b * 3 + c1) * 3 + j1) * a.L;
      fence_proxy_async_smem();
      mbar_expect_tx(&bar[nb1], gbytes);
      bulk_g2s(stg + nb1 * SB, G + (gb + l0) * a.KXS, gbytes, &bar[nb1]);
      if (nb1) ++issued1;
      else ++issued0;
    }
    if (!mbar_wait_or_flag(&bar[buf], (uint32_t)((t >> 1) & 1), a.wlim, failed)) broken = true;
    const float2* sg = stg + buf * SB;
    ct_fft_mapped_mid<float2, true, N, C, NT, EPT>(
        s, tw, tid,
        [&](int, int, int k, int col) -> float2 {
          const bool cj = 2 * k > N;
          const int kk = cj ? N - k : k;
          float2 A = make_float2(0.f, 0.f), B = make_float2(0.f, 0.f);
          if (kk <= ex) {
            const int ra = xp ? col : 2 * col, rb = xp ? col + C : 2 * col + 1;
            A = sg[ra * a.KXS + kk];
            B = sg[rb * a.KXS + kk];
            if (cj) { A.y = -A.y; B.y = -B.y; }
            if (k == 0) { A.y = 0.f; B.y = 0.f; }
          }
          return make_float2(A.x - B.y, A.y + B.x);
        },
        [&]() -> bool {   // the velocity tile of this j must have landed before the last stage
          if (!mbar_wait_or_flag(&bar[2], (uint32_t)(t & 1), a.wlim, failed)) broken = true;
          return true;
        },
        [&](int i, int q, int x, int col, float2 zv) {   // one paired fma for both lines
          acc[i][q] = __ffma2_rn(make_float2(us[col * TT::UP + x], us[(col + C) * TT::UP + x]), zv, acc[i][q]);
        });
    __syncthreads();   // s and the velocity tile are free
    if (tid == 0 && t + 1 < 9 && !broken) {   // once broken, issue nothing more
      const int j1 = (t + 1) % 3;
      fence_proxy_async_smem();
      mbar_expect_tx(&bar[2], (uint32_t)(2 * C * N * 4));
      const float* src = U + (long)j1 * Mtot + l0 * N;
      for (int r = 0; r < 2 * C; ++r)
        bulk_g2s(us + urow(r) * TT::UP, src + (long)r * N, (uint32_t)(N * 4), &bar[2]);
      ++issued2;
    }
    if (j == 2) {
      ct_fft_mapped<float2, false, N, C, NT, EPT>(
          s, tw, tid, [&](int i, int q, int, int) -> float2 { return acc[i][q]; },
          [&](int, int, int x, int col, float2 val) { s[swz(x, col, C)] = val; });
      __syncthreads();
      const long obase = ((long)b * 3 + c) * a.L;
      const float hs = 0.5f * a.so;
      // column fastest: a warp reads 4 whole swizzled rows of s (no bank conflicts) and writes
      // 32-byte runs of 8 lines
      for (int i = tid; i < C * a.KX; i += NT) {
        const int col = i % C, k = i / C;
        const long la = l0 + (xp ? col : 2 * col), lb = la + (xp ? C : 1);
        const float2 zk = s[swz(k, col, C)];
        const float2 zn = s[swz(k == 0 ? 0 : N - k, col, C)];
        out[(obase + la) * a.KXS + k] = make_float2((zk.x + zn.x) * hs, (zk.y - zn.y) * hs);
        out[(obase + lb) * a.KXS + k] = make_float2((zk.y + zn.y) * hs, (zn.x - zk.x) * hs);
      }
      __syncthreads();
    }
  }
  if (failed) atomicExch(err, 1);
  if (tid == 0) {   // no copy may still be landing when the block exits: the last issued phase of each
    mbar_wait_bounded(&bar[0], (uint32_t)((issued0 - 1) & 1), FIT_WAIT_CYCLES / 10);
    if (issued1 > 0) mbar_wait_bounded(&bar[1], (uint32_t)((issued1 - 1) & 1), FIT_WAIT_CYCLES / 10);
    mbar_wait_bounded(&bar[2], (uint32_t)((issued2 - 1) & 1), FIT_WAIT_CYCLES / 10);
  }
}

// ---- xmix, one independent thread group per complex column ---------------------------------------
// Same arithmetic as k_fz_xmix_reg for transform lengths whose schedule is three radix-8 stages
// (N = 512), with no block-wide barrier inside the pipeline: each complex column (a pair of lines)
// belongs to a group of N/8 threads (two warps at N = 512; one radix-8 butterfly per thread and
// stage) that syncs on its own named barrier and streams its own 2 gradient lines (double buffered)
// and its 2 velocity lines (single buffered, issued once the step's product has read the previous
// ones) by bulk copies on its own mbarriers. The 8 groups of a block share only the twiddle tables,
// so a group never waits for another group's progress.
// Column layout: row e = 64 e2 + 8 e1 + e0 of a 512-element column sits at
//   P(e) = 16 (e >> 4) + ((e0 ^ g) | (h << 3)),  g = (e1 >> 1) | ((e2 & 1) << 2),  h = (e1 ^ e2) & 1,
// a bijection inside each 16-row block. A half-warp's 16 eight-byte accesses then fall in 16
// different bank pairs in each of the stages' three access shapes: A, rows jt + 64q (32 consecutive
// rows per warp); B, rows 8 jt + q; C, rows 64 (jt >> 3) + (jt & 7) + 8q. No padding layout serves
// all three (one pad per 16 rows leaves C two-way conflicted). Each access is a per-thread base
// and a compile-time q: A at 64q + base(q & 1), B at base ^ q, C at (base ^ c(q)) + 16 (q >> 1).
// Twiddles of the middle stage as T1[q][k] = w^(8kq) and of the last stage as T2[q][j] = w^(jq), a
// warp's lanes reading consecutive entries; the values are the same table entries as
// k_fz_xmix_reg's.
template <int N>
struct XGTile {
  static constexpr int C = 8;          // columns (line pairs) per block
  static constexpr int G = N / 8;      // threads per column group
  static constexpr int NTHR = C * G;
  static constexpr bool OK = N == 512 && ct_nst(N) == 3 && ct_radix(N, 0) == 8 && ct_radix(N, 1) == 8 &&
                             ct_radix(N, 2) == 8;
  static constexpr int CP = N;                                       // column length (XOR layout)
  static constexpr size_t OFF_T1 = (size_t)C * CP * 8;
  static constexpr size_t OFF_T2 = OFF_T1 + 7 * 8 * 8;
  static constexpr size_t OFF_BAR = OFF_T2 + 7 * (size_t)G * 8;      // 3 mbarriers per group
  static constexpr size_t OFF_U = (OFF_BAR + 3 * C * 8 + 127) / 128 * 128;   // C x 2 velocity lines (floats)
  static constexpr size_t OFF_G = OFF_U + (size_t)C * 2 * N * 4;     // then 2 x C x (2 KX) complex
};

FIT_D void xg_bar(int id, int nthr) { asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(nthr) : "memory"); }

// P(e) of k_fz_xmix_grp's column layout
FIT_D int xg_swz(int e) {
  return (e & ~15) | (((e & 7) ^ (((e >> 4) & 3) | (((e >> 6) & 1) << 2))) | ((((e >> 3) ^ (e >> 6)) & 1) << 3));
}

// f(std::integral_constant<int, q>) for q = 0 .. Q-1, in order
template <int Q, class F>
FIT_D void xg_for(F&& f) {
  if constexpr (Q > 0) {
    xg_for<Q - 1>(f);
    f(std::integral_constant<int, Q - 1>{});
  }
}

// The float2 at shared byte address (base ^ X) + OFF. The XOR happens inside the access, so a
// shape keeps one base register instead of the compiler hoisting its eight XOR'd addresses out of
// the transform loop. Loads are ordered against the group barriers and the stores (all volatile).
template <int X, int OFF>
FIT_D float2 xg_ld(uint32_t base) {
  float2 v;
  if constexpr (X == 0)
    asm volatile("ld.shared.v2.f32 {%0, %1}, [%2+%3];" : "=f"(v.x), "=f"(v.y) : "r"(base), "n"(OFF));
  else
    asm volatile("{\n\t.reg .b32 xa;\n\txor.b32 xa, %2, %3;\n\tld.shared.v2.f32 {%0, %1}, [xa+%4];\n\t}"
                 : "=f"(v.x), "=f"(v.y) : "r"(base), "n"(X), "n"(OFF));
  return v;
}
template <int X, int OFF>
FIT_D void xg_st(uint32_t base, float2 v) {
  if constexpr (X == 0)
    asm volatile("st.shared.v2.f32 [%0+%1], {%2, %3};" ::"r"(base), "n"(OFF), "f"(v.x), "f"(v.y) : "memory");
  else
    asm volatile("{\n\t.reg .b32 xa;\n\txor.b32 xa, %0, %1;\n\tst.shared.v2.f32 [xa+%2], {%3, %4};\n\t}"
                 ::"r"(base), "n"(X), "n"(OFF), "f"(v.x), "f"(v.y) : "memory");
}

template <int N>
__global__ void __launch_bounds__(XGTile<N>::NTHR, 2) k_fz_xmix_grp(FzArgs a, const float2* __restrict__ G,
                                                                   const float* __restrict__ U,
                                                                   float2* __restrict__ out,
                                                                   const float2* __restrict__ twg, int* err) {
  typedef XGTile<N> TT;
  constexpr int GS = TT::G;            // threads per group = butterflies per stage
  constexpr int NR = N / 8;            // row stride of a radix-8 stage's inputs
  static_assert(GS == NR && NR == 64, "one radix-8 butterfly per thread and stage, N = 512");
  extern __shared__ __align__(128) unsigned char fit_smem_raw[];
  const int tid = threadIdx.x;
  const int g = tid / GS, jt = tid % GS;
  float2* s = reinterpret_cast<float2*>(fit_smem_raw) + (size_t)g * TT::CP;      // this group's column
  float2* T1 = reinterpret_cast<float2*>(fit_smem_raw + TT::OFF_T1);
  float2* T2 = reinterpret_cast<float2*>(fit_smem_raw + TT::OFF_T2);
  uint64_t* bar = reinterpret_cast<uint64_t*>(fit_smem_raw + TT::OFF_BAR) + 3 * g;   // gradient buffers 0, 1; velocity
  float* vbuf = reinterpret_cast<float*>(fit_smem_raw + TT::OFF_U) + (size_t)g * 2 * N;   // lines la, la + 1
  const int KX = a.KX, KXS = a.KXS;
  float2* gbuf = reinterpret_cast<float2*>(fit_smem_raw + TT::OFF_G) + (size_t)g * 2 * (2 * KXS);
  const uint32_t gbytes = (uint32_t)(2 * KXS) * 8u;
  const int b = blockIdx.x;
  const int ex = a.ext[b][0];
  const long Mtot = (long)N * N * N;
  const long la = (long)blockIdx.z * 2 * TT::C + 2 * g;   // this group's lines la, la + 1
  U += (long)a.uidx[b] * 3 * Mtot;
  const bool lead = jt == 0;
  const int gid = 1 + g;                                    // named barrier of the group
  for (int t = tid; t < 7 * 8; t += TT::NTHR) T1[t] = twg[(t % 8) * (t / 8 + 1) * (N / 64)];
  for (int t = tid; t < 7 * GS; t += TT::NTHR) T2[t] = twg[(t % GS) * (t / GS + 1)];
  if (lead) {
    mbar_init(&bar[0], 1);
    mbar_init(&bar[1], 1);
    mbar_init(&bar[2], 1);
    mbar_init_fence();
  }
  __syncthreads();   // the only block-wide barrier: twiddle tables and mbarriers ready
  if (lead) {
    mbar_expect_tx(&bar[0], gbytes);
    bulk_g2s(gbuf, G + (((long)b * 9) * a.L + la) * KXS, gbytes, &bar[0]);
    mbar_expect_tx(&bar[2], 2u * N * 4u);   // velocity lines of step 0 (j = 0), 4 KB contiguous
    bulk_g2s(vbuf, U + la * N, 2u * N * 4u, &bar[2]);
  }
  // per-thread bases of the three access shapes (l = jt & 7, u = jt >> 3): A, rows jt + 64q, at
  // 64q + aE (q even) or 64q + (aE ^ 12) (q odd: g gains bit 2, h flips); B, rows 8 jt + q, at
  // bB ^ q; C, rows 64u + l + 8q, at (cB ^ ((q >> 1) | ((q & 1) << 3))) + 16 (q >> 1)
  // (as shared byte addresses; the column starts on a 128-byte boundary, so XOR masks below 128
  // act on the element index alone)
  const int l = jt & 7, u = jt >> 3;
  const uint32_t s32 = smem_u32(s);
  const uint32_t aE = s32 + 8u * (16 * (u >> 1) + ((l ^ (u >> 1)) | ((u & 1) << 3)));
  const uint32_t bB = s32 + 8u * (16 * (4 * u + (l >> 1)) + (((l ^ u) & 1) << 3) + ((l >> 1) | ((u & 1) << 2)));
  const uint32_t cB = s32 + 8u * (64 * u + ((l ^ ((u & 1) << 2)) | ((u & 1) << 3)));
#define XG_LDA(q) xg_ld<((q) & 1) ? 96 : 0, 512 * (q)>(aE)
#define XG_STA(q, val) xg_st<((q) & 1) ? 96 : 0, 512 * (q)>(aE, val)
#define XG_STB(q, val) xg_st<8 * (q), 0>(bB, val)
#define XG_STC(q, val) xg_st<8 * (((q) >> 1) | (((q) & 1) << 3)), 128 * ((q) >> 1)>(cB, val)
  const int k1 = l;
  float2 t2r[7];   // this thread's last-stage twiddles w^(jt q), q = 1..7 (the same every step)
#pragma unroll
  for (int q = 0; q < 7; ++q) t2r[q] = T2[GS * q + jt];
  // waits as in k_fz_xmix_reg: a first wait that runs out flags the launch and is followed by a
  // full-bound wait; a thread whose second wait runs out is broken (the lead then issues nothing
  // more) and the group carries on with whatever the buffers hold, all indices data-independent
  bool failed = false, broken = false;
  int issued0 = 1, issued1 = 0, issued2 = 1;
  float2 acc[8];
  float2 v[8];
  for (int t = 0; t < 9; ++t) {
    const int c = t / 3, j = t % 3, buf = t & 1;
    if (j == 0) {
#pragma unroll
      for (int q = 0; q < 8; ++q) acc[q] = make_float2(0.f, 0.f);
    }
    if (lead && t + 1 < 9 && !broken) {   // next gradient lines into the other buffer (read at step t - 1)
      const int c1 = (t + 1) / 3, j1 = (t + 1) % 3, nb1 = (t + 1) & 1;
      fence_proxy_async_smem();
      mbar_expect_tx(&bar[nb1], gbytes);
      bulk_g2s(gbuf + nb1 * (2 * KXS), G + ((((long)b * 3 + c1) * 3 + j1) * a.L + la) * KXS, gbytes, &bar[nb1]);
      if (nb1) ++issued1;
      else ++issued0;
    }
    if (!mbar_wait_or_flag(&bar[buf], (uint32_t)((t >> 1) & 1), a.wlim, failed)) broken = true;
    // stage 0 of the inverse transform: inputs k = jt + 64q of the Hermitian pair z = A + iB
    const float2* ga = gbuf + buf * (2 * KXS);
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      const int k = jt + NR * q;
      const bool cj = 2 * k > N;
      const int kk = cj ? N - k : k;
      float2 A = make_float2(0.f, 0.f), B = make_float2(0.f, 0.f);
      if (kk <= ex) {
        A = ga[kk];
        B = ga[KXS + kk];
        if (cj) { A.y = -A.y; B.y = -B.y; }
        if (k == 0) { A.y = 0.f; B.y = 0.f; }
      }
      v[q] = make_float2(A.x - B.y, A.y + B.x);
    }
    dftr<float2, 8, true>(v);
    xg_for<8>([&](auto qc) { constexpr int q = decltype(qc)::value; XG_STB(q, v[q]); });
    xg_bar(gid, GS);
    // stage 1 (span 8)
    xg_for<8>([&](auto qc) {
      constexpr int q = decltype(qc)::value;
      float2 x = XG_LDA(q);
      if (q > 0 && k1 > 0) {
        float2 w = T1[8 * (q - 1) + k1];
        w.y = -w.y;
        x = cmul(x, w);
      }
      v[q] = x;
    });
    dftr<float2, 8, true>(v);
    xg_bar(gid, GS);
    xg_for<8>([&](auto qc) { constexpr int q = decltype(qc)::value; XG_STC(q, v[q]); });
    xg_bar(gid, GS);
    // stage 2 (span 64): outputs x = jt + 64q, accumulated against the velocity
    xg_for<8>([&](auto qc) {
      constexpr int q = decltype(qc)::value;
      float2 x = XG_LDA(q);
      if (q > 0) {
        float2 w = t2r[q - 1];
        w.y = -w.y;
        x = cmul(x, w);
      }
      v[q] = x;
    });
    dftr<float2, 8, true>(v);
    // the velocity at this thread's outputs x = jt + 64q of both lines, staged by the step's copy
    if (!mbar_wait_or_flag(&bar[2], (uint32_t)(t & 1), a.wlim, failed)) broken = true;
#pragma unroll
    for (int q = 0; q < 8; ++q)   // (acc.x, acc.y) += (u(la), u(la + 1)) * (v.x, v.y): one paired fma
      acc[q] = __ffma2_rn(make_float2(vbuf[jt + NR * q], vbuf[N + jt + NR * q]), v[q], acc[q]);
    xg_bar(gid, GS);   // the column and the velocity buffer are free
    if (lead && t + 1 < 9 && !broken) {   // the next step's velocity lines (read only after this barrier)
      fence_proxy_async_smem();
      mbar_expect_tx(&bar[2], 2u * N * 4u);
      bulk_g2s(vbuf, U + (long)((t + 1) % 3) * Mtot + la * N, 2u * N * 4u, &bar[2]);
      ++issued2;
    }
    if (j == 2) {   // forward transform of the product, kx <= K of both lines
#pragma unroll
      for (int q = 0; q < 8; ++q) v[q] = acc[q];
      dftr<float2, 8, false>(v);
      xg_for<8>([&](auto qc) { constexpr int q = decltype(qc)::value; XG_STB(q, v[q]); });
      xg_bar(gid, GS);
      xg_for<8>([&](auto qc) {
        constexpr int q = decltype(qc)::value;
        float2 x = XG_LDA(q);
        if (q > 0 && k1 > 0) x = cmul(x, T1[8 * (q - 1) + k1]);
        v[q] = x;
      });
      dftr<float2, 8, false>(v);
      xg_bar(gid, GS);
      xg_for<8>([&](auto qc) { constexpr int q = decltype(qc)::value; XG_STC(q, v[q]); });
      xg_bar(gid, GS);
      xg_for<8>([&](auto qc) {
        constexpr int q = decltype(qc)::value;
        float2 x = XG_LDA(q);
        if (q > 0) x = cmul(x, t2r[q - 1]);
        v[q] = x;
      });
      dftr<float2, 8, false>(v);
      xg_bar(gid, GS);   // every stage-2 read of the column is done before it is overwritten
      xg_for<8>([&](auto qc) { constexpr int q = decltype(qc)::value; XG_STA(q, v[q]); });   // Z(k), k = jt + 64q
      xg_bar(gid, GS);
      const long obase = ((long)b * 3 + c) * a.L;
      const float hs = 0.5f * a.so;
#pragma unroll
      for (int q = 0; q < 8; ++q) {
        const int k = jt + NR * q;
        if (k < KX) {
          const int e = k == 0 ? 0 : N - k;
          const float2 zk = v[q];
          const float2 zn = xg_ld<0, 0>(s32 + 8u * (uint32_t)xg_swz(e));
          out[(obase + la) * KXS + k] = make_float2((zk.x + zn.x) * hs, (zk.y - zn.y) * hs);
          out[(obase + la + 1) * KXS + k] = make_float2((zk.y + zn.y) * hs, (zn.x - zk.x) * hs);
        }
      }
      xg_bar(gid, GS);   // the column is free for the next transform
    }
  }
  if (failed) atomicExch(err, 1);
  if (lead) {   // no copy may still be landing when the block exits: the last issued phase of each
    mbar_wait_bounded(&bar[0], (uint32_t)((issued0 - 1) & 1), FIT_WAIT_CYCLES / 10);
    if (issued1 > 0) mbar_wait_bounded(&bar[1], (uint32_t)((issued1 - 1) & 1), FIT_WAIT_CYCLES / 10);
    mbar_wait_bounded(&bar[2], (uint32_t)((issued2 - 1) & 1), FIT_WAIT_CYCLES / 10);
  }
}
#undef XG_LDA
#undef XG_STA
#undef XG_STB
#undef XG_STC

// ---- yfwd --------------------------------------------------------------------------------------
template <int N>
__global__ void __launch_bounds__(FzTile<N>::NTHR, FzTile<N>::MINB) k_fz_yfwd(FzArgs a, const float2* __restrict__ in,
                                                                    float2* __restrict__ out,
                                                                    const float2* __restrict__ twg) {
  typedef FzTile<N> TT;
  constexpr bool PM = N == 512;   // permuted tile rows (see swzp) at 512 points
  constexpr int C = TT::C, E = TT::E, NT = TT::NTHR;
  extern __shared__ __align__(16) unsigned char fit_smem_raw[];
  float2* s = reinterpret_cast<float2*>(fit_smem_raw);
  float2* tw = s + E;
  const int tid = threadIdx.x;
  const int nkt = (a.KX + C - 1) / C;
  const int z = blockIdx.z / nkt, k0 = (blockIdx.z % nkt) * C;
  const int c = blockIdx.y, b = blockIdx.x;
  const long ib = ((long)b * 3 + c) * a.L + (long)N * z;
  // the twiddle table is first read after the transform's first stage, behind its block barrier
  for (int t = tid; t < N; t += NT) tw[t] = twg[t];
  const long obase = (((long)b * 3 + c) * N + z) * a.P1S;
  ct_fft_mapped<float2, false, N, C, NT, TT::EPT, false, PM>(
      s, tw, tid,
      [&](int, int, int e, int cc) -> float2 {
        const int kx = k0 + cc;
        return (kx < a.KX) ? in[(ib + e) * a.KXS + kx] : make_float2(0.f, 0.f);
      },
      [&](int, int, int e, int cc, float2 val) {
        const int kx = k0 + cc;
        const int f = fz_freq(e, N);
        if (kx < a.KX && f >= -a.K && f <= a.K) out[obase + (long)(f + a.K) * a.KX + kx] = val;
      });
}

// ---- zfwd + shell binning ------------------------------------------------------------------------
// After each component's transform, thread t reads the EPT contiguous kz rows
// [seg*EPT, seg*EPT + EPT) of pencil column t % C (seg = t / C): a warp covers two rows of all C
// columns per access (conflict-free under the swizzle), and along a pencil the shell index changes
// rarely, so each thread keeps a running (shell, sum) pair and flushes it to the block's FP64
// shared-memory bins only when the shell changes. The tile keeps the unpermuted row layout
// (swzp<false>): the eight transfer sums live across the three transforms, and the permuted
// layout's second address bases push the kernel further past 32 registers a thread.
template <int N>
__global__ void __launch_bounds__(FzTile<N>::NTHR, FzTile<N>::MINB_BIN) k_fz_zfwd_bin(FzArgs a, const float2* __restrict__ in,
                                                                        const float2* __restrict__ Ceff,
                                                                        const uint16_t* __restrict__ seff,
                                                                        double* __restrict__ partial,
                                                                        const float2* __restrict__ twg) {
  typedef FzTile<N> TT;
  constexpr int C = TT::C, E = TT::E, NT = TT::NTHR, EPT = TT::EPT;
  static_assert(NT * EPT == E && (NT / C) * EPT == N, "zfwd needs an exact thread/element split");
  extern __shared__ __align__(16) unsigned char fit_smem_raw[];
  float2* s = reinterpret_cast<float2*>(fit_smem_raw);
  float2* tw = s + E;
  double* bins = reinterpret_cast<double*>(tw + N);
  const int tid = threadIdx.x;
  const long c0 = (long)blockIdx.z * C;
  const int b = blockIdx.x;
  const int mycol = tid % C, seg = tid / C;
  const long col = c0 + mycol;
  for (int t = tid; t < N; t += NT) tw[t] = twg[t];
  for (int t = tid; t < a.nsh; t += NT) bins[t] = 0.0;
  float tacc[EPT];
#pragma unroll
  for (int r = 0; r < EPT; ++r) tacc[r] = 0.f;
  for (int c = 0; c < 3; ++c) {
    const long ib = ((long)b * 3 + c) * N;
    __syncthreads();
    ct_fft_mapped<float2, false, N, C, NT, EPT, false, false>(
        s, tw, tid,
        [&](int, int, int e, int cc) -> float2 {
          const long cl = c0 + cc;
          return (cl < a.P1) ? in[(ib + e) * a.P1S + cl] : make_float2(0.f, 0.f);
        },
        [&](int, int, int e, int cc, float2 val) { s[swzp<false>(e, cc, C)] = val; });
    __syncthreads();
#pragma unroll
    for (int r = 0; r < EPT; ++r) {
      const int e = seg * EPT + r;
      const int f = fz_freq(e, N);
      if (col < a.P1 && f >= -a.K && f <= a.K) {
        const float2 nv = s[swzp<false>(e, mycol, C)];
        const float2 cv = Ceff[((long)c * a.KY + f + a.K) * a.P1S + col];
        tacc[r] += cv.x * nv.x + cv.y * nv.y;
      }
    }
  }
  int cur = 0;
  double sum = 0.0;
#pragma unroll
  for (int r = 0; r < EPT; ++r) {
    const int e = seg * EPT + r;
    const int f = fz_freq(e, N);
    int sh = 0;
    if (col < a.P1 && f >= -a.K && f <= a.K) sh = seff[(long)(f + a.K) * a.P1S + col];
    if (sh != cur) {
      if (cur) atomicAdd(&bins[cur - 1], sum);
      cur = sh;
      sum = 0.0;
    }
    if (sh) sum += (double)tacc[r];
  }
  if (cur) atomicAdd(&bins[cur - 1], sum);
  __syncthreads();
  // partials laid out [mediator][shell][block] so that each shell's reduction reads contiguously
  double* pb = partial + (long)b * a.nsh * gridDim.z + blockIdx.z;
  for (int t = tid; t < a.nsh; t += NT) pb[(long)t * gridDim.z] = bins[t];
}

// The z-forward + shell-binning pass of a batch: one block per (mediator, pencil tile), block
// partials to partial[mediator][shell][tile].
template <int N>
int fz_zfwd_bin(const FzArgs& a, const float2* in, const float2* Ceff, const uint16_t* seff, double* partial,
                const float2* tw, cudaStream_t st) {
  typedef FzTile<N> TT;
  const size_t smb = TT::SMEM + sizeof(double) * a.nsh + 16;
  FIT_TRY(ct_prep_fused(k_fz_zfwd_bin<N>, smb, TT::NTHR));
  const unsigned pt = (unsigned)((a.P1 + TT::C - 1) / TT::C);
  k_fz_zfwd_bin<N><<<dim3(a.nb, 1, pt), TT::NTHR, smb, st>>>(a, in, Ceff, seff, partial, tw);
  FIT_LAUNCH_CHECK();
  return FIT_OK;
}

// ---- whole-box terms (partial fluxes) -------------------------------------------------------------
// z pass of a whole live box (no shell restriction): mediator b transforms field hidx[b] of H and
// its ik_z derivative; outputs as zinv's.
template <int N>
__global__ void __launch_bounds__(FzTile<N>::NTHR, FzTile<N>::MINB) k_fz_zinv_box(FzArgs a, const float2* __restrict__ H,
                                                                              const float* __restrict__ kd,
                                                                              float2* __restrict__ out,
                                                                              const float2* __restrict__ twg) {
  typedef FzTile<N> TT;
  constexpr bool PM = N == 512;   // permuted tile rows (see swzp) at 512 points
  constexpr int C = TT::C, E = TT::E, NT = TT::NTHR;
  extern __shared__ __align__(16) unsigned char fit_smem_raw[];
  float2* s = reinterpret_cast<float2*>(fit_smem_raw);
  float2* tw = s + E;
  const int tid = threadIdx.x;
  const long c0 = (long)blockIdx.z * C;
  const int c = blockIdx.y >> 1, v = blockIdx.y & 1, b = blockIdx.x;
  for (int t = tid; t < N; t += NT) tw[t] = twg[t];   // read after the transform's first barrier
  const float2* Hc = H + ((long)a.hidx[b] * 3 + c) * a.KY * a.P1;
  float2* ob = out + (((long)b * 3 + c) * 2 + v) * N * a.P1S;
  ct_fft_mapped<float2, true, N, C, NT, TT::EPT, false, PM>(
      s, tw, tid,
      [&](int, int, int e, int cc) -> float2 {
        const long col = c0 + cc;
        const int f = fz_freq(e, N);
        float2 val = make_float2(0.f, 0.f);
        if (col < a.P1 && f >= -a.K && f <= a.K) {
          const long m = (long)(f + a.K) * a.P1 + col;
          val = Hc[m];
          if (a.wbox) {
            const float w = a.wbox[(long)a.widx[b] * a.KY * a.P1 + m];
            val.x *= w;
            val.y *= w;
          }
          if (v) val = fz_muli(val, kd[f + a.K]);
        }
        return val;
      },
      [&](int, int, int e, int cc, float2 val) {
        const long col = c0 + cc;
        if (col < a.P1) ob[(long)e * a.P1S + col] = val;
      });
}

// forward z pass of yfwd's output, kept in the live box: out [b][c][kz'][col] (the nonlinear term)
template <int N>
__global__ void __launch_bounds__(FzTile<N>::NTHR, FzTile<N>::MINB) k_fz_zfwd_store(FzArgs a, const float2* __restrict__ in,
                                                                                float2* __restrict__ out,
                                                                                const float2* __restrict__ twg) {
  typedef FzTile<N> TT;
  constexpr bool PM = N == 512;   // permuted tile rows (see swzp) at 512 points
  constexpr int C = TT::C, E = TT::E, NT = TT::NTHR;
  extern __shared__ __align__(16) unsigned char fit_smem_raw[];
  float2* s = reinterpret_cast<float2*>(fit_smem_raw);
  float2* tw = s + E;
  const int tid = threadIdx.x;
  const long c0 = (long)blockIdx.z * C;
  const int c = blockIdx.y, b = blockIdx.x;
  for (int t = tid; t < N; t += NT) tw[t] = twg[t];   // read after the transform's first barrier
  const float2* ib = in + ((long)b * 3 + c) * N * a.P1S;
  float2* ob = out + ((long)b * 3 + c) * a.KY * a.P1;
  ct_fft_mapped<float2, false, N, C, NT, TT::EPT, false, PM>(
      s, tw, tid,
      [&](int, int, int e, int cc) -> float2 {
        const long col = c0 + cc;
        return (col < a.P1) ? ib[(long)e * a.P1S + col] : make_float2(0.f, 0.f);
      },
      [&](int, int, int e, int cc, float2 val) {
        const long col = c0 + cc;
        const int f = fz_freq(e, N);
        if (col < a.P1 && f >= -a.K && f <= a.K) ob[(long)(f + a.K) * a.P1 + col] = val;
      });
}

// ---- self-advecting velocity in physical space from H ------------------------------------------
// U = real(ifft3(Herm part of the masked velocity)) over the live box only: z pass of the KX x KY
// live pencils, y pass of the live kx columns, x pass two Hermitian lines per complex transform.
// Layouts: H [c][kz'][col] -> [c][z][col] -> [c][z][y][kx] -> U [c][z][y][x].
template <int N>
__global__ void __launch_bounds__(FzTile<N>::NTHR, FzTile<N>::MINB) k_fz_uz(FzArgs a, const float2* __restrict__ H,
                                                                          float2* __restrict__ out,
                                                                          const float2* __restrict__ twg) {
  typedef FzTile<N> TT;
  constexpr bool PM = N == 512;   // permuted tile rows (see swzp) at 512 points
  constexpr int C = TT::C, E = TT::E, NT = TT::NTHR;
  extern __shared__ __align__(16) unsigned char fit_smem_raw[];
  float2* s = reinterpret_cast<float2*>(fit_smem_raw);
  float2* tw = s + E;
  const int tid = threadIdx.x;
  const long c0 = (long)blockIdx.y * C;
  const int c = blockIdx.x;
  for (int t = tid; t < N; t += NT) tw[t] = twg[t];   // read after the transform's first barrier
  const float2* Hc = H + (long)c * a.KY * a.P1;
  float2* oc = out + (long)c * N * a.P1;
  ct_fft_mapped<float2, true, N, C, NT, TT::EPT, false, PM>(
      s, tw, tid,
      [&](int, int, int e, int cc) -> float2 {
        const long col = c0 + cc;
        const int f = fz_freq(e, N);
        return (col < a.P1 && f >= -a.K && f <= a.K) ? Hc[(long)(f + a.K) * a.P1 + col] : make_float2(0.f, 0.f);
      },
      [&](int, int, int e, int cc, float2 val) {
        const long col = c0 + cc;
        if (col < a.P1) oc[(long)e * a.P1 + col] = val;
      });
}

template <int N>
__global__ void __launch_bounds__(FzTile<N>::NTHR, FzTile<N>::MINB) k_fz_uy(FzArgs a, const float2* __restrict__ in,
                                                                          float2* __restrict__ out,
                                                                          const float2* __restrict__ twg) {
  typedef FzTile<N> TT;
  constexpr bool PM = N == 512;   // permuted tile rows (see swzp) at 512 points
  constexpr int C = TT::C, E = TT::E, NT = TT::NTHR;
  extern __shared__ __align__(16) unsigned char fit_smem_raw[];
  float2* s = reinterpret_cast<float2*>(fit_smem_raw);
  float2* tw = s + E;
  const int tid = threadIdx.x;
  const int nkt = (a.KX + C - 1) / C;
  const int z = blockIdx.y / nkt, k0 = (blockIdx.y % nkt) * C, c = blockIdx.x;
  for (int t = tid; t < N; t += NT) tw[t] = twg[t];   // read after the transform's first barrier
  const float2* ib = in + ((long)c * N + z) * a.P1;
  float2* ob = out + ((long)c * N + z) * N * a.KX;
  ct_fft_mapped<float2, true, N, C, NT, TT::EPT, false, PM>(
      s, tw, tid,
      [&](int, int, int e, int cc) -> float2 {
        const int kx = k0 + cc;
        const int f = fz_freq(e, N);
        return (kx < a.KX && f >= -a.K && f <= a.K) ? ib[kx + (long)a.KX * (f + a.K)] : make_float2(0.f, 0.f);
      },
      [&](int, int, int e, int cc, float2 val) {
        const int kx = k0 + cc;
        if (kx < a.KX) ob[(long)e * a.KX + kx] = val;
      });
}

template <int N>
__global__ void __launch_bounds__(FzTile<N>::NTHR, FzTile<N>::MINB) k_fz_ux(FzArgs a, const float2* __restrict__ in,
                                                                          float* __restrict__ out,
                                                                          const float2* __restrict__ twg, float scale) {
  typedef FzTile<N> TT;
  constexpr bool PM = N == 512;   // permuted tile rows (see swzp) at 512 points
  constexpr int C = TT::C, E = TT::E, NT = TT::NTHR;
  extern __shared__ __align__(16) unsigned char fit_smem_raw[];
  float2* s = reinterpret_cast<float2*>(fit_smem_raw);
  float2* tw = s + E;
  const int tid = threadIdx.x;
  const long l0 = (long)blockIdx.x * 2 * C;   // lines of all three components, 2C per block
  for (int t = tid; t < N; t += NT) tw[t] = twg[t];   // read after the transform's first barrier
  ct_fft_mapped<float2, true, N, C, NT, TT::EPT, false, PM>(
      s, tw, tid,
      [&](int, int, int k, int col) -> float2 {
        const bool cj = 2 * k > N;
        const int kk = cj ? N - k : k;
        float2 A = make_float2(0.f, 0.f), B = make_float2(0.f, 0.f);
        if (kk <= a.K) {   // |kx| <= K < N / 2: the self-conjugate bin N / 2 never holds data
          A = in[(l0 + 2 * col) * a.KX + kk];
          B = in[(l0 + 2 * col + 1) * a.KX + kk];
          if (cj) { A.y = -A.y; B.y = -B.y; }
          if (k == 0) { A.y = 0.f; B.y = 0.f; }
        }
        return make_float2(A.x - B.y, A.y + B.x);
      },
      [&](int, int, int x, int col, float2 zv) {
        out[(l0 + 2 * col) * N + x] = zv.x * scale;
        out[(l0 + 2 * col + 1) * N + x] = zv.y * scale;
      });
}

// Raise the dynamic shared-memory limit and size the carveout for the kernel's occupancy.
template <typename K>
static int ct_prep_fused(K kern, size_t smem, int nthr) {
  static std::mutex mu;
  static std::unordered_map<const void*, size_t> done;   // kernels already prepared, by footprint
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

// Line pairing of the x pass with the fewer shared-memory bank conflicts on the gradient tile:
// a half-warp reads 8-byte elements at rows row(c) of stride KX (the tile's row stride, KXS) for its columns c = lane % C and
// consecutive positions lane / C; the busiest bank's distinct-word count is compared.
static int fz_xpair(int KX, int C) {
  int best = 0, best_hits = 1 << 30;
  for (int mode = 0; mode < 2; ++mode) {
    int words[16], hits = 0;
    for (int lane = 0; lane < 16; ++lane) {
      const int c = lane % C, j = lane / C;
      words[lane] = 2 * ((mode ? c : 2 * c) * KX + j);
    }
    for (int bank = 0; bank < 32; ++bank) {
      int distinct[32], nd = 0;
      for (int lane = 0; lane < 16; ++lane)
        for (int h = 0; h < 2; ++h) {
          const int w = words[lane] + h;
          if (w % 32 != bank) continue;
          bool seen = false;
          for (int t = 0; t < nd; ++t) seen = seen || distinct[t] == w;
          if (!seen) distinct[nd++] = w;
        }
      if (nd > hits) hits = nd;
    }
    if (hits < best_hits) best_hits = hits, best = mode;
  }
  return best;
}

// ---- host launcher of the velocity passes (instantiated per transform length) --------------------
// bufZ holds 3 N P1 and bufY 3 N^2 KX complex values; U receives 3 N^3 floats scaled by `scale`.
template <int N>
int fz_velocity(const FzArgs& a, const float2* H, float2* bufZ, float2* bufY, float* U, const float2* tw, float scale,
                cudaStream_t st) {
  typedef FzTile<N> TT;
  constexpr int C = TT::C;
  FIT_TRY(ct_prep_fused(k_fz_uz<N>, TT::SMEM, TT::NTHR));
  FIT_TRY(ct_prep_fused(k_fz_uy<N>, TT::SMEM, TT::NTHR));
  FIT_TRY(ct_prep_fused(k_fz_ux<N>, TT::SMEM, TT::NTHR));
  const unsigned pt = (unsigned)((a.P1 + C - 1) / C);
  const unsigned nkt = (unsigned)((a.KX + C - 1) / C);
  const double cpx = 8.0, L = (double)N * N;
  fit_prof_begin(PK_S2S_VELOCITY, cpx * 3.0 * (a.KY + (double)N) * a.P1, st);
  k_fz_uz<N><<<dim3(3, pt), TT::NTHR, TT::SMEM, st>>>(a, H, bufZ, tw);
  fit_prof_end(st);
  FIT_LAUNCH_CHECK();
  fit_prof_begin(PK_S2S_VELOCITY, cpx * 3.0 * ((double)N * a.P1 + L * a.KX), st);
  k_fz_uy<N><<<dim3(3, nkt * N), TT::NTHR, TT::SMEM, st>>>(a, bufZ, bufY, tw);
  fit_prof_end(st);
  FIT_LAUNCH_CHECK();
  fit_prof_begin(PK_S2S_VELOCITY, 3.0 * L * (cpx * a.KX + 4.0 * N), st);
  k_fz_ux<N><<<(unsigned)(3 * a.L / (2 * C)), TT::NTHR, TT::SMEM, st>>>(a, bufY, U, tw, scale);
  fit_prof_end(st);
  FIT_LAUNCH_CHECK();
  return FIT_OK;
}

// ---- the x pass of a batch: register-accumulating form where its tiles fit, else staged ---------
template <int N>
int fz_xpass(const FzArgs& a, const float2* G, const float* U, float2* out, const float2* tw, int* err,
             cudaStream_t st) {
  typedef FzTile<N> TT;
  constexpr int C = TT::C;
  typedef XTile<N> XT;
  const size_t smx = XT::SMEM_FIXED + 2 * (size_t)(2 * XT::C * a.KXS) * 8;
  const bool bulk = smx <= 227 * 1024 && (a.L % (2 * XT::C)) == 0;   // 16-byte alignment holds: L, 2C are multiples of 16
  typedef XRTile<N> XR;
  const size_t smr = XR::OFF_G + 2 * (size_t)(2 * XR::C * a.KXS) * 8;
  const char* env = getenv("FIT_XMIX_BULK");   // selects the previous form of the x pass
  bool reg = XR::OK && bulk && smr <= 227 * 1024 && !(env && env[0] == '1');
  FzArgs aw = a;
  aw.wlim = fit_wait_cycles();
  typedef XGTile<N> XG;
  const char* envr = getenv("FIT_XMIX_REG");   // selects the block-synchronous register form
  if constexpr (XG::OK) {
    const size_t smg = XG::OFF_G + 2 * (size_t)XG::C * (2 * a.KXS) * 8;
    if (reg && !(envr && envr[0] == '1') && smg <= 227 * 1024 && (a.L % (2 * XG::C)) == 0) {
      FIT_TRY(ct_prep_fused(k_fz_xmix_grp<N>, smg, XG::NTHR));
      k_fz_xmix_grp<N><<<dim3(a.nb, 1, (unsigned)(a.L / (2 * XG::C))), XG::NTHR, smg, st>>>(aw, G, U, out, tw, err);
      FIT_LAUNCH_CHECK();
      return FIT_OK;
    }
  }
  if constexpr (XR::OK) {
    if (reg) {
      FIT_TRY(ct_prep_fused(k_fz_xmix_reg<N>, smr, XR::NTHR));
      FzArgs ax = aw;
      ax.xpair = fz_xpair(a.KXS, XR::C);
      k_fz_xmix_reg<N><<<dim3(a.nb, 1, (unsigned)(a.L / (2 * XR::C))), XR::NTHR, smr, st>>>(ax, G, U, out, tw, err);
    }
  }
  if (reg) {
  } else if (bulk) {
    FIT_TRY(ct_prep_fused(k_fz_xmix_bulk<N>, smx, XT::NTHR));
    k_fz_xmix_bulk<N><<<dim3(a.nb, 1, (unsigned)(a.L / (2 * XT::C))), XT::NTHR, smx, st>>>(aw, G, U, out, tw, err);
  } else {
    FIT_TRY(ct_prep_fused(k_fz_xmix<N>, TT::SMEM, TT::NTHR));
    k_fz_xmix<N><<<dim3(a.nb, 1, (unsigned)((a.L + 2 * C - 1) / (2 * C))), TT::NTHR, TT::SMEM, st>>>(a, G, U, out,
                                                                                                     tw);
  }
  FIT_LAUNCH_CHECK();
  return FIT_OK;
}

// ---- host launcher for a batch of whole-box nonlinear terms (instantiated per transform length) ---
// Mediator b: N_b = (u_{uidx[b]} . grad) f_{hidx[b]} over the whole live box (a.ext all K), written
// to Nout [b][c][kz'][col]. Scratch as fz_batch.
template <int N>
int fz_terms(const FzArgs& a, const float2* H, const float* kd, const float* U, float2* bufA, float2* bufB,
             float2* Nout, const float2* tw, int* err, cudaStream_t st) {
  typedef FzTile<N> TT;
  constexpr int C = TT::C;
  const size_t sm = TT::SMEM;
  FIT_TRY(ct_prep_fused(k_fz_zinv_box<N>, sm, TT::NTHR));
  FIT_TRY(ct_prep_fused(k_fz_yinv<N>, sm, TT::NTHR));
  FIT_TRY(ct_prep_fused(k_fz_xmix<N>, sm, TT::NTHR));
  FIT_TRY(ct_prep_fused(k_fz_yfwd<N>, sm, TT::NTHR));
  FIT_TRY(ct_prep_fused(k_fz_zfwd_store<N>, sm, TT::NTHR));
  const unsigned pt = (unsigned)((a.P1 + C - 1) / C);
  const unsigned nkt = (unsigned)((a.KX + C - 1) / C);
  const double cpx = 8.0, L = (double)N * N;
  fit_prof_begin(PK_S2S_ZINV, cpx * a.nb * (3.0 * a.KY * a.P1 + 6.0 * N * a.P1), st);
  k_fz_zinv_box<N><<<dim3(a.nb, 6, pt), TT::NTHR, sm, st>>>(a, H, kd, bufA, tw);
  fit_prof_end(st);
  FIT_LAUNCH_CHECK();
  fit_prof_begin(PK_S2S_YINV, cpx * a.nb * (6.0 * N * a.P1 + 9.0 * L * a.KX), st);
  FIT_TRY(fz_yinv<N>(a, bufA, kd, bufB, tw, err, N, st));
  fit_prof_end(st);
  fit_prof_begin(PK_S2S_XMIX, cpx * a.nb * (9.0 * L * a.KX + 3.0 * L * a.KX) + 4.0 * 3.0 * N * L * 2, st);
  FIT_TRY(fz_xpass<N>(a, bufB, U, bufA, tw, err, st));
  fit_prof_end(st);
  fit_prof_begin(PK_S2S_YFWD, cpx * a.nb * (3.0 * L * a.KX + 3.0 * N * a.P1), st);
  k_fz_yfwd<N><<<dim3(a.nb, 3, nkt * N), TT::NTHR, sm, st>>>(a, bufA, bufB, tw);
  fit_prof_end(st);
  FIT_LAUNCH_CHECK();
  fit_prof_begin(PK_S2S_ZFWD_BIN, cpx * a.nb * (3.0 * N * a.P1 + 3.0 * a.KY * a.P1), st);
  k_fz_zfwd_store<N><<<dim3(a.nb, 3, pt), TT::NTHR, sm, st>>>(a, bufB, Nout, tw);
  fit_prof_end(st);
  FIT_LAUNCH_CHECK();
  return FIT_OK;
}

// ---- zinv of a batch over pencil tiles [t0, t1) (the rest of the batch then runs with nozinv) ----
template <int N>
int fz_zinv_tiles(const FzArgs& a, const float2* H, const float* kd, float2* bufA, const float2* tw, int t0, int t1,
                  cudaStream_t st) {
  typedef FzTile<N> TT;
  const size_t sm = TT::SMEM;
  FIT_TRY(ct_prep_fused(k_fz_zinv<N>, sm, TT::NTHR));
  if (t1 <= t0 || a.nb < 1) return FIT_OK;
  const int pt = (int)((a.P1 + TT::C - 1) / TT::C);
  double zin_b = 0.0;   // the tile range's share of the batch's algorithmic bytes (as in fz_batch)
  for (int b = 0; b < a.nb; ++b) {
    const double ex = a.ext[b][0], ey = a.ext[b][1], ez = a.ext[b][2];
    const double Pm = (ex + 1.0) * (2.0 * ey + 1.0);
    zin_b += 8.0 * 6.0 * N * Pm + 2.0 * (2.0 * ez + 1.0) * Pm;
  }
  FzArgs ar = a;
  ar.tz0 = t0;
  fit_prof_begin(PK_S2S_ZINV, zin_b * (t1 - t0) / pt, st);
  k_fz_zinv<N><<<dim3(a.nb, 6, t1 - t0), TT::NTHR, sm, st>>>(ar, H, kd, bufA, tw);
  fit_prof_end(st);
  FIT_LAUNCH_CHECK();
  return FIT_OK;
}

// ---- host launcher for one batch (instantiated per transform length) -------------------------
template <int N>
int fz_batch(const FzArgs& a, const float2* H, const float2* Ceff, const uint16_t* seff,
             const float* kd, const float* U, float2* bufA, float2* bufB, double* partial, const float2* tw,
             int* err, cudaStream_t st) {
  typedef FzTile<N> TT;
  constexpr int C = TT::C;
  const size_t sm = TT::SMEM;
  FIT_TRY(ct_prep_fused(k_fz_zinv<N>, sm, TT::NTHR));
  FIT_TRY(ct_prep_fused(k_fz_yinv<N>, sm, TT::NTHR));
  FIT_TRY(ct_prep_fused(k_fz_xmix<N>, sm, TT::NTHR));
  FIT_TRY(ct_prep_fused(k_fz_yfwd<N>, sm, TT::NTHR));
  const unsigned pt = (unsigned)((a.P1 + C - 1) / C);
  const unsigned nkt = (unsigned)((a.KX + C - 1) / C);
  const double cpx = 8.0;
  // algorithmic bytes of the pruned passes (lower bounds of what they move): mediator b has
  // Pm = (ex+1)(2ey+1) live pencils; zinv reads the band map on 2ez+1 z frequencies of each (the
  // velocity itself only on the shell's own modes, not counted) and writes 6 N-long outputs; yinv
  // reads the 6 zinv outputs of those pencils once and writes 9 outputs of N x N x (ex+1) values
  double zin_b = 0.0, yin_b = 0.0;
  for (int b = 0; b < a.nb; ++b) {
    const double ex = a.ext[b][0], ey = a.ext[b][1], ez = a.ext[b][2];
    const double Pm = (ex + 1.0) * (2.0 * ey + 1.0);
    zin_b += cpx * 6.0 * N * Pm + 2.0 * (2.0 * ez + 1.0) * Pm;
    yin_b += cpx * (6.0 * N * Pm + 9.0 * (double)N * N * (ex + 1.0));
  }
  if (!a.nozinv) {
    fit_prof_begin(PK_S2S_ZINV, zin_b, st);
    k_fz_zinv<N><<<dim3(a.nb, 6, pt), TT::NTHR, sm, st>>>(a, H, kd, bufA, tw);
    fit_prof_end(st);
    FIT_LAUNCH_CHECK();
  }
  fit_prof_begin(PK_S2S_YINV, yin_b, st);
  FIT_TRY(fz_yinv<N>(a, bufA, kd, bufB, tw, err, N, st));
  fit_prof_end(st);
  fit_prof_begin(PK_S2S_XMIX,
                 cpx * a.nb * (9.0 * (double)N * N * a.KX + 3.0 * (double)N * N * a.KX) + 4.0 * 3.0 * N * N * N, st);
  FIT_TRY(fz_xpass<N>(a, bufB, U, bufA, tw, err, st));
  fit_prof_end(st);
  fit_prof_begin(PK_S2S_YFWD, cpx * a.nb * (3.0 * (double)N * N * a.KX + 3.0 * N * a.P1), st);
  k_fz_yfwd<N><<<dim3(a.nb, 3, nkt * N), TT::NTHR, sm, st>>>(a, bufA, bufB, tw);
  fit_prof_end(st);
  FIT_LAUNCH_CHECK();
  fit_prof_begin(PK_S2S_ZFWD_BIN, cpx * (a.nb * 3.0 * N * a.P1 + 3.0 * a.KY * a.P1) + 2.0 * a.KY * a.P1, st);
  FIT_TRY(fz_zfwd_bin<N>(a, bufB, Ceff, seff, partial, tw, st));
  fit_prof_end(st);
  return FIT_OK;
}

}  // namespace fit
