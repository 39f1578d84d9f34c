// Learned subfilter-stress closure: a pointwise MLP 9 -> 64 -> 64 -> 6 (ReLU), BF16 operands on the
// tensor cores (mma.sync m16n8k16, FP32 accumulation).
//
// Parameters are one FP32 buffer (the optimizer's master copy); every block converts them to BF16
// in shared memory when it starts. Layout (floats):
//   W1[64][16] (inputs padded 9 -> 16), b1[64], W2[64][64], b2[64], W3[8][64] (outputs padded 6 -> 8), b3[8]
// Point data is field-major with field stride ld >= P: X[f*ld + p] (9 features: the filtered
// velocity-gradient tensor A_ij = d_j ū_i, f = 3i + j), T/Y[o*ld + p] (6 stress components
// tau_00 tau_11 tau_22 tau_01 tau_02 tau_12), so a slab of points is a pointer offset. Features are
// multiplied by in_scale[f] and targets by t_scale[o] before the network sees them; the forward
// entry point divides its outputs by t_scale again.
//
// Fragment layouts of mma.m16n8k16 (g = lane/4, t = lane%4): A a0 (g, 2t..2t+1), a1 (g+8, 2t..),
// a2 (g, 2t+8..), a3 (g+8, 2t+8..); B b0 (k 2t..2t+1, n g), b1 (k 2t+8.., n g); C c0 (g, 2t),
// c1 (g, 2t+1), c2 (g+8, 2t), c3 (g+8, 2t+1). Two adjacent n8 accumulator tiles form the A operand
// of the next layer's k16 step, so the forward pass chains layers in registers.
#include <cuda_bf16.h>
#include <stdint.h>
#include <stdlib.h>

#include "fit_common.cuh"
#include "fit_umma.cuh"

#define MLP_IN 16
#define MLP_H 64
#define MLP_OUT 8
#define MLP_NPARAM (64 * 16 + 64 + 64 * 64 + 64 + 8 * 64 + 8)

namespace fit {

struct MlpOff {
  static constexpr int W1 = 0, B1 = 1024, W2 = 1088, B2 = 5184, W3 = 5248, B3 = 5760;
};

FIT_D uint32_t pack_bf16(float lo, float hi) {
  __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
  return *reinterpret_cast<uint32_t*>(&v);
}

FIT_D float2 unpack_bf16(uint32_t u) {
  __nv_bfloat162 v = *reinterpret_cast<__nv_bfloat162*>(&u);
  return __bfloat1622float2(v);
}

FIT_D void mma_bf16(float* d, const uint32_t* a, uint32_t b0, uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// BF16 weights in shared memory: forward operands W1[64][16], W2[64][64], W3[8][64] (k contiguous),
// backward operands W2T[64][64] (W2 transposed), W3T[64][16] (W3 transposed, outputs padded to 16).
struct MlpSmem {
  __nv_bfloat16 W1[64 * 16], W2[64 * 64], W3[8 * 64], W2T[64 * 64], W3T[64 * 16];
  float b1[64], b2[64], b3[8];
};

FIT_D void mlp_load_weights(MlpSmem* w, const float* __restrict__ P, int tid, int nthr) {
  for (int i = tid; i < 64 * 16; i += nthr) w->W1[i] = __float2bfloat16_rn(P[MlpOff::W1 + i]);
  for (int i = tid; i < 64 * 64; i += nthr) {
    const int r = i / 64, c = i % 64;
    const __nv_bfloat16 v = __float2bfloat16_rn(P[MlpOff::W2 + i]);
    w->W2[i] = v;
    w->W2T[c * 64 + r] = v;
  }
  for (int i = tid; i < 8 * 64; i += nthr) {
    const int r = i / 64, c = i % 64;
    w->W3[i] = __float2bfloat16_rn(P[MlpOff::W3 + i]);
    w->W3T[c * 16 + r] = w->W3[i];
  }
  for (int i = tid; i < 64 * 8; i += nthr) w->W3T[(i / 8) * 16 + 8 + (i % 8)] = __float2bfloat16_rn(0.f);
  for (int i = tid; i < 64; i += nthr) {
    w->b1[i] = P[MlpOff::B1 + i];
    w->b2[i] = P[MlpOff::B2 + i];
  }
  for (int i = tid; i < 8; i += nthr) w->b3[i] = P[MlpOff::B3 + i];
}

FIT_D uint32_t ld32(const __nv_bfloat16* p) { return *reinterpret_cast<const uint32_t*>(p); }

// Forward of one 16-point tile held by one warp. x: A fragment of the scaled inputs.
// Returns layer outputs: h1a/h2a (BF16 A fragments, 4 k-steps), y (C fragment, 8 outputs).
FIT_D void mlp_tile_forward(const MlpSmem* w, const uint32_t* xa, uint32_t h1a[4][4], uint32_t h2a[4][4],
                            float* y, int lane) {
  const int g = lane >> 2, t = lane & 3;
  float acc[8][4];
#pragma unroll
  for (int n = 0; n < 8; ++n) {
    const float bb0 = w->b1[n * 8 + 2 * t], bb1 = w->b1[n * 8 + 2 * t + 1];
    acc[n][0] = bb0; acc[n][1] = bb1; acc[n][2] = bb0; acc[n][3] = bb1;
    const __nv_bfloat16* wr = w->W1 + (n * 8 + g) * 16;
    mma_bf16(acc[n], xa, ld32(wr + 2 * t), ld32(wr + 2 * t + 8));
  }
#pragma unroll
  for (int s = 0; s < 4; ++s) {
    const float* lo = acc[2 * s];
    const float* hi = acc[2 * s + 1];
    h1a[s][0] = pack_bf16(fmaxf(lo[0], 0.f), fmaxf(lo[1], 0.f));
    h1a[s][1] = pack_bf16(fmaxf(lo[2], 0.f), fmaxf(lo[3], 0.f));
    h1a[s][2] = pack_bf16(fmaxf(hi[0], 0.f), fmaxf(hi[1], 0.f));
    h1a[s][3] = pack_bf16(fmaxf(hi[2], 0.f), fmaxf(hi[3], 0.f));
  }
#pragma unroll
  for (int n = 0; n < 8; ++n) {
    const float bb0 = w->b2[n * 8 + 2 * t], bb1 = w->b2[n * 8 + 2 * t + 1];
    acc[n][0] = bb0; acc[n][1] = bb1; acc[n][2] = bb0; acc[n][3] = bb1;
#pragma unroll
    for (int s = 0; s < 4; ++s) {
      const __nv_bfloat16* wr = w->W2 + (n * 8 + g) * 64 + 16 * s;
      mma_bf16(acc[n], h1a[s], ld32(wr + 2 * t), ld32(wr + 2 * t + 8));
    }
  }
#pragma unroll
  for (int s = 0; s < 4; ++s) {
    const float* lo = acc[2 * s];
    const float* hi = acc[2 * s + 1];
    h2a[s][0] = pack_bf16(fmaxf(lo[0], 0.f), fmaxf(lo[1], 0.f));
    h2a[s][1] = pack_bf16(fmaxf(lo[2], 0.f), fmaxf(lo[3], 0.f));
    h2a[s][2] = pack_bf16(fmaxf(hi[0], 0.f), fmaxf(hi[1], 0.f));
    h2a[s][3] = pack_bf16(fmaxf(hi[2], 0.f), fmaxf(hi[3], 0.f));
  }
  const float bb0 = w->b3[2 * t], bb1 = w->b3[2 * t + 1];
  y[0] = bb0; y[1] = bb1; y[2] = bb0; y[3] = bb1;
#pragma unroll
  for (int s = 0; s < 4; ++s) {
    const __nv_bfloat16* wr = w->W3 + g * 64 + 16 * s;
    mma_bf16(y, h2a[s], ld32(wr + 2 * t), ld32(wr + 2 * t + 8));
  }
}

// A fragment of 16 points x 16 features (9 real) from field-major X, scaled, BF16. In the
// homogeneous form the scaled features v are divided by |v| (s = |v|^2 returned per row g / g+8):
// the network sees the direction of the gradient tensor and its output is multiplied by s, so the
// predicted stress is homogeneous of degree 2 in A, like the exact subfilter stress at leading
// order (tau ~ ell^2/12 A A^T for a Gaussian filter).
// raw (optional): the unscaled features this lane loaded, [row][col group][pair].
FIT_D void mlp_load_x(const float* __restrict__ X, long ld, long P, long p0, const float* sc, uint32_t* xa,
                      int lane, bool homog, float* s, float (*raw)[2][2] = nullptr) {
  const int g = lane >> 2, t = lane & 3;
  float v[2][2][2];   // [row g / g+8][col group 2t / 2t+8][pair]
#pragma unroll
  for (int r = 0; r < 2; ++r)
#pragma unroll
    for (int cg = 0; cg < 2; ++cg)
#pragma unroll
      for (int e = 0; e < 2; ++e) {
        const int f = 2 * t + 8 * cg + e;
        const long p = p0 + g + 8 * r;
        const float x = (f < 9 && p < P) ? X[(long)f * ld + p] : 0.f;
        if (raw) raw[r][cg][e] = x;
        v[r][cg][e] = x * sc[f < 9 ? f : 0];
      }
#pragma unroll
  for (int r = 0; r < 2; ++r) {
    float q = v[r][0][0] * v[r][0][0] + v[r][0][1] * v[r][0][1] + v[r][1][0] * v[r][1][0] + v[r][1][1] * v[r][1][1];
    q += __shfl_xor_sync(0xffffffffu, q, 1);   // the quad of lanes holding row g (g+8)
    q += __shfl_xor_sync(0xffffffffu, q, 2);
    s[r] = homog ? q : 1.f;
    if (homog) {
      const float inv = q > 0.f ? 1.f / sqrtf(q) : 0.f;
#pragma unroll
      for (int cg = 0; cg < 2; ++cg)
#pragma unroll
        for (int e = 0; e < 2; ++e) v[r][cg][e] *= inv;
    }
  }
  xa[0] = pack_bf16(v[0][0][0], v[0][0][1]);
  xa[1] = pack_bf16(v[1][0][0], v[1][0][1]);
  xa[2] = pack_bf16(v[0][1][0], v[0][1][1]);
  xa[3] = pack_bf16(v[1][1][0], v[1][1][1]);
}

// The nine features of the point of row r, gathered from the quad of lanes that loaded them
// (lane t holds features 2t, 2t+1 and, for t = 0, feature 8).
FIT_D void quad_features(const float (*raw)[2][2], int r, int lane, float* A) {
  const int q0 = lane & ~3;
#pragma unroll
  for (int f = 0; f < 8; ++f) {
    const float mine = (f & 1) ? raw[r][0][1] : raw[r][0][0];
    A[f] = __shfl_sync(0xffffffffu, mine, q0 | (f >> 1));
  }
  A[8] = __shfl_sync(0xffffffffu, raw[r][1][0], q0);
}

// Gradient-model stress (below) and Pi = -tau_ij S_ij, S = (A + A^T)/2 (the closure's flux, fused
// epilogue), on a point's features held in registers.
FIT_D float gradient_model_stress_r(int o, const float* A) {
  const int i = o < 3 ? o : (o == 5 ? 1 : 0), j = o < 3 ? o : (o == 3 ? 1 : 2);
  float t = 0.f;
#pragma unroll
  for (int k = 0; k < 3; ++k) t += A[3 * i + k] * A[3 * j + k];
  return t;
}
FIT_D float stress_dot_strain_r(int o, float tau, const float* A) {
  const int i = o < 3 ? o : (o == 5 ? 1 : 0), j = o < 3 ? o : (o == 3 ? 1 : 2);
  if (i == j) return -tau * A[3 * i + i];
  return -tau * (A[3 * i + j] + A[3 * j + i]);
}

// Gradient-model stress component o (00 11 22 01 02 12) without its ell^2/12 factor: sum_k A_ik A_jk.
FIT_D float gradient_model_stress(int o, const float* __restrict__ X, long ld, long p) {
  const int i = o < 3 ? o : (o == 5 ? 1 : 0), j = o < 3 ? o : (o == 3 ? 1 : 2);
  float t = 0.f;
#pragma unroll
  for (int k = 0; k < 3; ++k) t += X[(long)(3 * i + k) * ld + p] * X[(long)(3 * j + k) * ld + p];
  return t;
}

__global__ void __launch_bounds__(256) k_mlp_forward(const float* __restrict__ Pm, const float* __restrict__ X,
                                                     long ld, long P, const float* __restrict__ in_scale,
                                                     const float* __restrict__ t_scale, float* __restrict__ Y,
                                                     float* __restrict__ Pi, int homog, float clark) {
  __shared__ MlpSmem w;
  __shared__ float sc[9], osc[6];
  mlp_load_weights(&w, Pm, threadIdx.x, blockDim.x);
  if (threadIdx.x < 9) sc[threadIdx.x] = in_scale[threadIdx.x];
  if (threadIdx.x < 6) osc[threadIdx.x] = 1.f / t_scale[threadIdx.x];
  __syncthreads();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  const int g = lane >> 2, t = lane & 3;
  const long ntile = (P + 15) / 16;
  for (long tile = (long)blockIdx.x * nw + warp; tile < ntile; tile += (long)gridDim.x * nw) {
    const long p0 = tile * 16;
    uint32_t xa[4], h1a[4][4], h2a[4][4];
    float y[4], sn[2], raw[2][2][2];
    mlp_load_x(X, ld, P, p0, sc, xa, lane, homog != 0, sn, raw);
    mlp_tile_forward(&w, xa, h1a, h2a, y, lane);
#pragma unroll
    for (int r = 0; r < 2; ++r) {
      const long p = p0 + g + 8 * r;
      float A[9];
      quad_features(raw, r, lane, A);
      float part = 0.f;
#pragma unroll
      for (int e = 0; e < 2; ++e) {
        const int o = 2 * t + e;
        if (o < 6 && p < P) {
          float tau = y[2 * r + e] * sn[r] * osc[o];
          if (clark != 0.f) tau += clark * gradient_model_stress_r(o, A);
          if (Y) Y[(long)o * ld + p] = tau;
          if (Pi) part += stress_dot_strain_r(o, tau, A);
        }
      }
      // the four lanes of a quad hold the six outputs of point p
      part += __shfl_xor_sync(0xffffffffu, part, 1);
      part += __shfl_xor_sync(0xffffffffu, part, 2);
      if (Pi && t == 0 && p < P) Pi[p] = part;
    }
  }
}

// ---- forward on the fifth-generation tensor cores (tcgen05) ---------------------------------------
// One CTA of 128 threads handles 128 points per tile, one point per thread (tensor-memory lane =
// thread). Each layer is D = A * W^T with M = 128: the A tile (BF16, canonical K-major layout) is
// written to shared memory by the threads, thread 0 issues the MMAs (K = 16 steps) and commits
// them to an mbarrier, every thread waits on it (clock-bounded) and reads its accumulator row from
// tensor memory. Layer widths: 16 (9 features) -> 64 -> 64 -> 16 (6 outputs). The 64 tensor-memory
// columns are reused by all three layers (each accumulator is read out before the next MMA).
// The biases ride in the MMAs: columns 9 and 10 of the layer-1 A tile hold ones, and each bias b is
// split into BF16 parts hi = bf16(b), lo = bf16(b - hi) placed in those columns of a weight tile
// (W1 itself for layer 1; one K = 16 step of A1 against the bias tiles B2b / B3b for layers 2 and 3,
// whose other columns are zero), so the accumulator leaves the tensor cores as W x + b with b exact
// to about 2^-17 of |b|. The epilogue then only rounds to BF16 pairs and applies the ReLU on the
// packed pairs (relu and rounding commute), about half the instructions per point of an epilogue
// that adds the bias and clamps in FP32.
struct MlpTcSmem {
  __nv_bfloat16 W1[64 * 16], W2[64 * 64], W3[16 * 64], A1[128 * 16], A2[128 * 64];   // canonical layouts
  __nv_bfloat16 B2b[64 * 16], B3b[16 * 16];   // bias tiles of layers 2 and 3 (columns 9, 10)
  float sc[9], osc[6];
  uint64_t bar;
  uint32_t tmem;
};

FIT_D void st_chunk(__nv_bfloat16* tile, uint32_t off, const float* v) {   // 8 BF16 values, 16 bytes
  *reinterpret_cast<uint4*>(reinterpret_cast<char*>(tile) + off) =
      make_uint4(pack_bf16(v[0], v[1]), pack_bf16(v[2], v[3]), pack_bf16(v[4], v[5]), pack_bf16(v[6], v[7]));
}

FIT_D void st_bf16_at(__nv_bfloat16* tile, uint32_t off, float v) {
  *reinterpret_cast<__nv_bfloat16*>(reinterpret_cast<char*>(tile) + off) = __float2bfloat16_rn(v);
}

// The BF16 parts of a bias value: hi = bf16(b), lo = bf16(b - hi).
FIT_D void bias_split(float b, float* hi, float* lo) {
  const float h = __bfloat162float(__float2bfloat16_rn(b));
  *hi = h;
  *lo = b - h;
}

// relu(D) of this thread's 64-column accumulator row (bias included) -> its row of the next layer's
// A tile: BF16 pairs, clamped as pairs.
FIT_D void hidden_to_a(uint32_t tl, __nv_bfloat16* A2, int row) {
  const __nv_bfloat162 zero = __floats2bfloat162_rn(0.f, 0.f);
#pragma unroll
  for (int c4 = 0; c4 < 4; ++c4) {
    float d[16];
    tmem_ld16(tl + 16 * c4, d);
    uint32_t w[8];
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      __nv_bfloat162 v = __hmax2(__floats2bfloat162_rn(d[2 * i], d[2 * i + 1]), zero);
      w[i] = *reinterpret_cast<uint32_t*>(&v);
    }
    *reinterpret_cast<uint4*>(reinterpret_cast<char*>(A2) + umma_off(row, 16 * c4, 64)) = make_uint4(w[0], w[1], w[2], w[3]);
    *reinterpret_cast<uint4*>(reinterpret_cast<char*>(A2) + umma_off(row, 16 * c4 + 8, 64)) =
        make_uint4(w[4], w[5], w[6], w[7]);
  }
}

__global__ void __launch_bounds__(128) k_mlp_forward_tc(const float* __restrict__ Pm, const float* __restrict__ X,
                                                        long ld, long P, const float* __restrict__ in_scale,
                                                        const float* __restrict__ t_scale, float* __restrict__ Y,
                                                        float* __restrict__ Pi, int homog, float clark, int* err,
                                                        long long wlim) {
  extern __shared__ __align__(128) unsigned char mlp_tc_raw[];
  MlpTcSmem& S = *reinterpret_cast<MlpTcSmem*>(mlp_tc_raw);
  const int tid = threadIdx.x, warp = tid >> 5;
  for (int i = tid; i < 64 * 16; i += 128) {   // W1 with b1 in columns 9 (hi) and 10 (lo)
    const int r = i / 16, c = i % 16;
    float w = Pm[MlpOff::W1 + i];
    if (c == 9 || c == 10) {
      float hi, lo;
      bias_split(Pm[MlpOff::B1 + r], &hi, &lo);
      w = c == 9 ? hi : lo;
    }
    st_bf16_at(S.W1, umma_off(r, c, 16), w);
  }
  for (int i = tid; i < 64 * 64; i += 128) st_bf16_at(S.W2, umma_off(i / 64, i % 64, 64), Pm[MlpOff::W2 + i]);
  for (int i = tid; i < 16 * 64; i += 128)   // outputs padded 8 -> 16 rows (rows 6.. never read out)
    st_bf16_at(S.W3, umma_off(i / 64, i % 64, 64), i < 8 * 64 ? Pm[MlpOff::W3 + i] : 0.f);
  for (int i = tid; i < 64 * 16; i += 128) {   // bias tiles: b2, b3 split into columns 9 and 10
    const int r = i / 16, c = i % 16;
    float hi, lo;
    bias_split(Pm[MlpOff::B2 + r], &hi, &lo);
    st_bf16_at(S.B2b, umma_off(r, c, 16), c == 9 ? hi : (c == 10 ? lo : 0.f));
    if (r < 16) {
      bias_split(r < 8 ? Pm[MlpOff::B3 + r] : 0.f, &hi, &lo);
      st_bf16_at(S.B3b, umma_off(r, c, 16), c == 9 ? hi : (c == 10 ? lo : 0.f));
    }
  }
  if (tid < 9) S.sc[tid] = in_scale[tid];
  if (tid < 6) S.osc[tid] = 1.f / t_scale[tid];
  if (tid == 0) {
    mbar_init(&S.bar, 1);
    mbar_init_fence();
  }
  if (warp == 0) {
    tmem_alloc(&S.tmem, 64);
    tmem_relinquish();
  }
  fence_proxy_async_smem();   // weights written by the threads, read by the tensor cores
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tbase = S.tmem;
  const uint32_t tl = tbase + ((uint32_t)(warp * 32) << 16);   // this warp's 32 lanes
  const uint32_t aA1 = smem_u32(S.A1), aA2 = smem_u32(S.A2);
  const uint32_t aW1 = smem_u32(S.W1), aW2 = smem_u32(S.W2), aW3 = smem_u32(S.W3);
  const uint32_t aB2 = smem_u32(S.B2b), aB3 = smem_u32(S.B3b);
  constexpr uint32_t ID64 = umma_idesc_bf16(128, 64), ID16 = umma_idesc_bf16(128, 16);
  uint32_t phase = 0;
  bool failed = false;
  auto wait_mma = [&]() {
    mbar_wait_or_flag(&S.bar, phase, wlim, failed);   // a second, full-bound wait keeps phases in step
    phase ^= 1u;
    tc_fence_after();
  };
  auto publish_a = [&]() {   // A tile rows written by the threads -> visible to the MMA issue
    fence_proxy_async_smem();
    tc_fence_before();
    __syncthreads();
  };
  const long ntile = (P + 127) / 128;
  float An[9];   // features of this thread's point in the next tile, loaded a tile ahead
  {
    const long p = (long)blockIdx.x * 128 + tid;
#pragma unroll
    for (int f = 0; f < 9; ++f) An[f] = p < P ? X[(long)f * ld + p] : 0.f;
  }
  for (long tile = blockIdx.x; tile < ntile; tile += gridDim.x) {
    const long p = tile * 128 + tid;
    const bool live = p < P;
    float A[9], v[16];
#pragma unroll
    for (int f = 0; f < 9; ++f) A[f] = An[f];
    {   // the loads of the next tile overlap this tile's MMA chain
      const long pn = p + (long)gridDim.x * 128;
#pragma unroll
      for (int f = 0; f < 9; ++f) An[f] = pn < P ? X[(long)f * ld + pn] : 0.f;
    }
    float q = 0.f;
#pragma unroll
    for (int f = 0; f < 16; ++f) {
      v[f] = f < 9 ? A[f] * S.sc[f] : 0.f;
      q += v[f] * v[f];
    }
    const float sn = homog ? q : 1.f;
    if (homog) {   // the network sees the direction of the scaled gradient tensor
      const float inv = q > 0.f ? 1.f / sqrtf(q) : 0.f;
#pragma unroll
      for (int f = 0; f < 9; ++f) v[f] *= inv;
    }
    v[9] = 1.f;    // the bias columns
    v[10] = 1.f;
    st_chunk(S.A1, umma_off(tid, 0, 16), v);
    st_chunk(S.A1, umma_off(tid, 8, 16), v + 8);
    publish_a();
    if (tid == 0) {
      tc_fence_after();
      umma_bf16(tbase, umma_desc(aA1, 128, 256), umma_desc(aW1, 128, 256), ID64, false);
      umma_commit(&S.bar);
    }
    wait_mma();
    hidden_to_a(tl, S.A2, tid);
    publish_a();
    if (tid == 0) {
      tc_fence_after();
      umma_bf16(tbase, umma_desc(aA1, 128, 256), umma_desc(aB2, 128, 256), ID64, false);   // b2 (ones x bias)
#pragma unroll
      for (int s = 0; s < 4; ++s)
        umma_bf16(tbase, umma_desc(aA2 + 256 * s, 128, 1024), umma_desc(aW2 + 256 * s, 128, 1024), ID64, true);
      umma_commit(&S.bar);
    }
    wait_mma();
    hidden_to_a(tl, S.A2, tid);   // layer 2 has read A2: its MMAs completed
    publish_a();
    if (tid == 0) {
      tc_fence_after();
      umma_bf16(tbase, umma_desc(aA1, 128, 256), umma_desc(aB3, 128, 256), ID16, false);   // b3
#pragma unroll
      for (int s = 0; s < 4; ++s)
        umma_bf16(tbase, umma_desc(aA2 + 256 * s, 128, 1024), umma_desc(aW3 + 256 * s, 128, 1024), ID16, true);
      umma_commit(&S.bar);
    }
    wait_mma();
    float y[16];
    tmem_ld16(tl, y);
    if (live) {
      float part = 0.f;
#pragma unroll
      for (int o = 0; o < 6; ++o) {
        float tau = y[o] * sn * S.osc[o];
        if (clark != 0.f) tau += clark * gradient_model_stress_r(o, A);
        if (Y) Y[(long)o * ld + p] = tau;
        part += stress_dot_strain_r(o, tau, A);
      }
      if (Pi) Pi[p] = part;
    }
    tc_fence_before();
    __syncthreads();   // accumulator columns and the A tiles are free for the next tile
    tc_fence_after();
  }
  if (failed) atomicExch(err, 1);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (warp == 0) tmem_dealloc(tbase, 64);
}

// ---- training step on tcgen05 -------------------------------------------------------------------
// One CTA of 128 threads per SM walks tiles of 128 points (one point per thread and tensor-memory
// lane). Per tile, six MMA rounds: the three forward layers, dH2 = dY W3, dH1 = dZ2 W2 (M = 128,
// point-major A tiles), then the weight gradients, which reduce over the points (K = 128) and
// therefore read point-contiguous ("transposed") tiles written column-wise by the threads:
//   G2: [dZ2T; dZ1T] x H1T -> rows 0..63 = dW2[h2][h1]
//   G1: [dZ2T; dZ1T] x XT' -> rows 64..127 = dW1[h1][f] (f < 9) and db1 (f = 9: XT' row 9 is ones)
//   G3: [H2T; dZ2T] x dYT' -> rows 0..63 = dW3[o][h2] transposed (o < 6), rows 64..127 col 8 = db2
//        (dYT' row 8 is ones)
// H2T, dZ2T and dZ1T are consecutive 64-row blocks of one tile, so both stacked A operands are
// plain descriptors. The gradient accumulators stay in tensor memory across the CTA's tiles and
// are added to grad once; db3 and the loss are reduced on the CUDA cores. ReLU masks of H1 and H2
// are kept as 64-bit registers per point.
struct MlpTrainTcSmem {
  __nv_bfloat16 W1[64 * 16], W2[64 * 64], W3[16 * 64], W2T[64 * 64], W3T[64 * 16];   // canonical layouts
  __nv_bfloat16 A1[128 * 16];    // layer-1 A tile, then dY (point-major, K = 16)
  __nv_bfloat16 A2[128 * 64];    // H1, H2, then dZ2 (point-major)
  __nv_bfloat16 XT[16 * 128];    // features (rows 0..8), ones (row 9), point-contiguous
  __nv_bfloat16 H1T[64 * 128];
  __nv_bfloat16 ST[192 * 128];   // H2T | dZ2T | dZ1T
  __nv_bfloat16 dYT[16 * 128];   // dY (rows 0..5), ones (row 8)
  float b1[64], b2[64], b3[8], sc[9], tsc[6], db3[8];
  double lsum[4];
  uint64_t bar;
  uint32_t tmem;
};

FIT_D void st_col(__nv_bfloat16* tile, int row, int p, float v) {   // element (row, point p), K = 128
  st_bf16_at(tile, umma_off(row, p, 128), v);
}

__global__ void __launch_bounds__(128, 1) k_mlp_train_tc(const float* __restrict__ Pm, const float* __restrict__ X,
                                                         const float* __restrict__ T, long ld, long P, long Ptot,
                                                         const float* __restrict__ in_scale,
                                                         const float* __restrict__ t_scale, float* __restrict__ grad,
                                                         double* __restrict__ loss, int homog, int* err,
                                                         long long wlim) {
  extern __shared__ __align__(128) unsigned char mlp_tr_raw[];
  MlpTrainTcSmem& S = *reinterpret_cast<MlpTrainTcSmem*>(mlp_tr_raw);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  for (int i = tid; i < 64 * 16; i += 128) st_bf16_at(S.W1, umma_off(i / 16, i % 16, 16), Pm[MlpOff::W1 + i]);
  for (int i = tid; i < 64 * 64; i += 128) {
    const int r = i / 64, c = i % 64;
    const float w = Pm[MlpOff::W2 + i];
    st_bf16_at(S.W2, umma_off(r, c, 64), w);
    st_bf16_at(S.W2T, umma_off(c, r, 64), w);
  }
  for (int i = tid; i < 16 * 64; i += 128) {   // W3 padded to 16 output rows; W3T[h][o], o padded to 16
    const int r = i / 64, c = i % 64;
    const float w = r < 8 ? Pm[MlpOff::W3 + i] : 0.f;
    st_bf16_at(S.W3, umma_off(r, c, 64), w);
    st_bf16_at(S.W3T, umma_off(c, r, 16), w);
  }
  for (int i = tid; i < 16 * 128; i += 128) {   // constant rows of XT' and dYT'
    const int r = i / 128, p = i % 128;
    st_col(S.XT, r, p, r == 9 ? 1.f : 0.f);
    st_col(S.dYT, r, p, r == 8 ? 1.f : 0.f);
  }
  if (tid < 64) {
    S.b1[tid] = Pm[MlpOff::B1 + tid];
    S.b2[tid] = Pm[MlpOff::B2 + tid];
  }
  if (tid < 8) {
    S.b3[tid] = Pm[MlpOff::B3 + tid];
    S.db3[tid] = 0.f;
  }
  if (tid < 9) S.sc[tid] = in_scale[tid];
  if (tid < 6) S.tsc[tid] = t_scale[tid];
  if (tid == 0) {
    mbar_init(&S.bar, 1);
    mbar_init_fence();
  }
  if (warp == 0) {
    tmem_alloc(&S.tmem, 256);
    tmem_relinquish();
  }
  fence_proxy_async_smem();
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tbase = S.tmem;
  const uint32_t tl = tbase + ((uint32_t)(warp * 32) << 16);
  const uint32_t TD = tbase, TG2 = tbase + 64, TG1 = tbase + 128, TG3 = tbase + 144;   // column bases
  const uint32_t aA1 = smem_u32(S.A1), aA2 = smem_u32(S.A2), aXT = smem_u32(S.XT), aH1T = smem_u32(S.H1T);
  const uint32_t aST = smem_u32(S.ST), adYT = smem_u32(S.dYT);
  const uint32_t aW1 = smem_u32(S.W1), aW2 = smem_u32(S.W2), aW3 = smem_u32(S.W3);
  const uint32_t aW2T = smem_u32(S.W2T), aW3T = smem_u32(S.W3T);
  constexpr uint32_t ID64 = umma_idesc_bf16(128, 64), ID16 = umma_idesc_bf16(128, 16);
  __nv_bfloat16* H2T = S.ST;
  __nv_bfloat16* dZ2T = S.ST + 64 * 128;
  __nv_bfloat16* dZ1T = S.ST + 128 * 128;
  uint32_t phase = 0;
  bool failed = false;
  auto wait_mma = [&]() {
    mbar_wait_or_flag(&S.bar, phase, wlim, failed);   // a second, full-bound wait keeps phases in step
    phase ^= 1u;
    tc_fence_after();
  };
  auto publish = [&]() {
    fence_proxy_async_smem();
    tc_fence_before();
    __syncthreads();
  };
  const float inv = 2.f / (float)Ptot;
  double lsum = 0.0;
  float db3[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
  bool first = true;
  const long ntile = (P + 127) / 128;
  for (long tile = blockIdx.x; tile < ntile; tile += gridDim.x) {
    const long p = tile * 128 + tid;
    const bool live = p < P;
    // (a) features -> A1 row and XT column
    float v[16];
    float q = 0.f;
#pragma unroll
    for (int f = 0; f < 16; ++f) {
      v[f] = (f < 9 && live) ? X[(long)f * ld + p] * S.sc[f] : 0.f;
      q += v[f] * v[f];
    }
    const float sn = homog ? q : 1.f;
    if (homog) {
      const float iq = q > 0.f ? 1.f / sqrtf(q) : 0.f;
#pragma unroll
      for (int f = 0; f < 16; ++f) v[f] *= iq;
    }
    st_chunk(S.A1, umma_off(tid, 0, 16), v);
    st_chunk(S.A1, umma_off(tid, 8, 16), v + 8);
#pragma unroll
    for (int f = 0; f < 9; ++f) st_col(S.XT, f, tid, v[f]);
    publish();
    if (tid == 0) {
      tc_fence_after();
      umma_bf16(TD, umma_desc(aA1, 128, 256), umma_desc(aW1, 128, 256), ID64, false);
      umma_commit(&S.bar);
    }
    wait_mma();
    // (b) H1 = relu(D + b1): A2 row, H1T column, mask
    uint32_t m1[2] = {0u, 0u}, m2[2] = {0u, 0u};
#pragma unroll
    for (int c4 = 0; c4 < 4; ++c4) {
      float d[16];
      tmem_ld16(tl + 16 * c4, d);
#pragma unroll
      for (int i = 0; i < 16; ++i) {
        const int h = 16 * c4 + i;
        d[i] = fmaxf(d[i] + S.b1[h], 0.f);
        if (d[i] > 0.f) m1[h >> 5] |= 1u << (h & 31);
        st_col(S.H1T, h, tid, d[i]);
      }
      st_chunk(S.A2, umma_off(tid, 16 * c4, 64), d);
      st_chunk(S.A2, umma_off(tid, 16 * c4 + 8, 64), d + 8);
    }
    publish();
    if (tid == 0) {
      tc_fence_after();
#pragma unroll
      for (int k = 0; k < 4; ++k)
        umma_bf16(TD, umma_desc(aA2 + 256 * k, 128, 1024), umma_desc(aW2 + 256 * k, 128, 1024), ID64, k > 0);
      umma_commit(&S.bar);
    }
    wait_mma();
    // (c) H2 = relu(D + b2): A2 row (layer 2 has read H1), H2T column, mask
#pragma unroll
    for (int c4 = 0; c4 < 4; ++c4) {
      float d[16];
      tmem_ld16(tl + 16 * c4, d);
#pragma unroll
      for (int i = 0; i < 16; ++i) {
        const int h = 16 * c4 + i;
        d[i] = fmaxf(d[i] + S.b2[h], 0.f);
        if (d[i] > 0.f) m2[h >> 5] |= 1u << (h & 31);
        st_col(H2T, h, tid, d[i]);
      }
      st_chunk(S.A2, umma_off(tid, 16 * c4, 64), d);
      st_chunk(S.A2, umma_off(tid, 16 * c4 + 8, 64), d + 8);
    }
    publish();
    if (tid == 0) {
      tc_fence_after();
#pragma unroll
      for (int k = 0; k < 4; ++k)
        umma_bf16(TD, umma_desc(aA2 + 256 * k, 128, 1024), umma_desc(aW3 + 256 * k, 128, 1024), ID16, k > 0);
      umma_commit(&S.bar);
    }
    wait_mma();
    // (d) loss and dY = 2 (s y - t T) s / Ptot: A1 row (point-major), dYT column
    {
      float y[16], dy[16];
      tmem_ld16(tl, y);
#pragma unroll
      for (int o = 0; o < 16; ++o) {
        float d = 0.f;
        if (o < 6 && live) {
          const float diff = (y[o] + S.b3[o]) * sn - T[(long)o * ld + p] * S.tsc[o];
          lsum += (double)diff * diff;
          d = inv * diff * sn;
        }
        dy[o] = __bfloat162float(__float2bfloat16_rn(d));   // the value the MMAs see
      }
#pragma unroll
      for (int o = 0; o < 6; ++o) {
        db3[o] += dy[o];
        st_col(S.dYT, o, tid, dy[o]);
      }
      st_chunk(S.A1, umma_off(tid, 0, 16), dy);
      st_chunk(S.A1, umma_off(tid, 8, 16), dy + 8);
    }
    publish();
    if (tid == 0) {
      tc_fence_after();
      umma_bf16(TD, umma_desc(aA1, 128, 256), umma_desc(aW3T, 128, 256), ID64, false);
      umma_commit(&S.bar);
    }
    wait_mma();
    // (e) dZ2 = dH2 * (H2 > 0): A2 row (layer 3 has read H2), dZ2T column
#pragma unroll
    for (int c4 = 0; c4 < 4; ++c4) {
      float d[16];
      tmem_ld16(tl + 16 * c4, d);
#pragma unroll
      for (int i = 0; i < 16; ++i) {
        const int h = 16 * c4 + i;
        d[i] = (m2[h >> 5] >> (h & 31)) & 1u ? d[i] : 0.f;
        st_col(dZ2T, h, tid, d[i]);
      }
      st_chunk(S.A2, umma_off(tid, 16 * c4, 64), d);
      st_chunk(S.A2, umma_off(tid, 16 * c4 + 8, 64), d + 8);
    }
    publish();
    if (tid == 0) {
      tc_fence_after();
#pragma unroll
      for (int k = 0; k < 4; ++k)
        umma_bf16(TD, umma_desc(aA2 + 256 * k, 128, 1024), umma_desc(aW2T + 256 * k, 128, 1024), ID64, k > 0);
      umma_commit(&S.bar);
    }
    wait_mma();
    // (f) dZ1 = dH1 * (H1 > 0): dZ1T column
#pragma unroll
    for (int c4 = 0; c4 < 4; ++c4) {
      float d[16];
      tmem_ld16(tl + 16 * c4, d);
#pragma unroll
      for (int i = 0; i < 16; ++i) {
        const int h = 16 * c4 + i;
        st_col(dZ1T, h, tid, (m1[h >> 5] >> (h & 31)) & 1u ? d[i] : 0.f);
      }
    }
    publish();
    // (g) weight gradients, accumulated over the CTA's tiles in tensor memory
    if (tid == 0) {
      tc_fence_after();
      const uint32_t aS2 = aST + 8 * 2048;   // dZ2T: the stack [dZ2T; dZ1T]
#pragma unroll
      for (int k = 0; k < 8; ++k) {
        const bool acc = !first || k > 0;
        umma_bf16(TG2, umma_desc(aS2 + 256 * k, 128, 2048), umma_desc(aH1T + 256 * k, 128, 2048), ID64, acc);
        umma_bf16(TG1, umma_desc(aS2 + 256 * k, 128, 2048), umma_desc(aXT + 256 * k, 128, 2048), ID16, acc);
        umma_bf16(TG3, umma_desc(aST + 256 * k, 128, 2048), umma_desc(adYT + 256 * k, 128, 2048), ID16, acc);
      }
      umma_commit(&S.bar);
    }
    wait_mma();   // the tiles read by the gradient MMAs are rewritten by the next tile
    first = false;
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
  }
  // flush: loss and db3 on the CUDA cores, the tensor-memory gradients by their owning threads
  for (int o = 16; o > 0; o >>= 1) lsum += __shfl_down_sync(0xffffffffu, lsum, o);
#pragma unroll
  for (int o = 0; o < 6; ++o) {
    float sdb = db3[o];
    for (int k = 16; k > 0; k >>= 1) sdb += __shfl_down_sync(0xffffffffu, sdb, k);
    if (lane == 0) atomicAdd(&S.db3[o], sdb);
  }
  if (lane == 0) S.lsum[warp] = lsum;
  if (!first) {   // this CTA processed at least one tile
    if (warp < 2) {   // lanes 0..63: dW2 rows h2, dW3^T rows h2
      const int h2 = tid;
#pragma unroll
      for (int c4 = 0; c4 < 4; ++c4) {
        float d[16];
        tmem_ld16(tl + 64 + 16 * c4, d);
#pragma unroll
        for (int i = 0; i < 16; ++i) atomicAdd(&grad[MlpOff::W2 + h2 * 64 + 16 * c4 + i], d[i]);
      }
      float d[16];
      tmem_ld16(tl + 144, d);
#pragma unroll
      for (int o = 0; o < 6; ++o) atomicAdd(&grad[MlpOff::W3 + o * 64 + h2], d[o]);
    } else {   // lanes 64..127: dW1 rows h1 with db1, db2
      const int h = tid - 64;
      float d[16];
      tmem_ld16(tl + 128, d);
#pragma unroll
      for (int f = 0; f < 9; ++f) atomicAdd(&grad[MlpOff::W1 + h * 16 + f], d[f]);
      atomicAdd(&grad[MlpOff::B1 + h], d[9]);
      tmem_ld16(tl + 144, d);
      atomicAdd(&grad[MlpOff::B2 + h], d[8]);
    }
  }
  if (failed) atomicExch(err, 1);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (tid < 6) atomicAdd(&grad[MlpOff::B3 + tid], S.db3[tid]);
  if (tid == 0) atomicAdd(loss, S.lsum[0] + S.lsum[1] + S.lsum[2] + S.lsum[3]);
  if (warp == 0) tmem_dealloc(tbase, 256);
}

// ---- training: fused forward + backward, weight gradients reduced over points by MMAs --------------
// A block of 4 warps handles 64 points per iteration (16 per warp). Activations are staged in shared
// memory transposed (feature-major, 64 points contiguous) so that the weight-gradient products
// dW = dZ^T H (reduction over points) read their operands as 32-bit pairs.
struct MlpTrainSmem {
  __nv_bfloat16 XT[16 * 64], H1T[64 * 64], H2T[64 * 64], dYT[16 * 64], dH1T[64 * 64], dH2T[64 * 64];
};

FIT_D void st_c_transposed(__nv_bfloat16* base, int ld, int col0, int row0, const float* c, int lane) {
  // C fragment (16 points x 8 features starting at feature col0) -> base[feature][row0 + point]
  const int g = lane >> 2, t = lane & 3;
  base[(col0 + 2 * t) * ld + row0 + g] = __float2bfloat16_rn(c[0]);
  base[(col0 + 2 * t + 1) * ld + row0 + g] = __float2bfloat16_rn(c[1]);
  base[(col0 + 2 * t) * ld + row0 + g + 8] = __float2bfloat16_rn(c[2]);
  base[(col0 + 2 * t + 1) * ld + row0 + g + 8] = __float2bfloat16_rn(c[3]);
}

FIT_D void st_a_transposed(__nv_bfloat16* base, int ld, int col0, int row0, const uint32_t* a, int lane) {
  // A fragment (16 points x 16 features starting at col0) -> base[feature][row0 + point]
  const int g = lane >> 2, t = lane & 3;
  const float2 v0 = unpack_bf16(a[0]), v1 = unpack_bf16(a[1]), v2 = unpack_bf16(a[2]), v3 = unpack_bf16(a[3]);
  base[(col0 + 2 * t) * ld + row0 + g] = __float2bfloat16_rn(v0.x);
  base[(col0 + 2 * t + 1) * ld + row0 + g] = __float2bfloat16_rn(v0.y);
  base[(col0 + 2 * t) * ld + row0 + g + 8] = __float2bfloat16_rn(v1.x);
  base[(col0 + 2 * t + 1) * ld + row0 + g + 8] = __float2bfloat16_rn(v1.y);
  base[(col0 + 2 * t + 8) * ld + row0 + g] = __float2bfloat16_rn(v2.x);
  base[(col0 + 2 * t + 9) * ld + row0 + g] = __float2bfloat16_rn(v2.y);
  base[(col0 + 2 * t + 8) * ld + row0 + g + 8] = __float2bfloat16_rn(v3.x);
  base[(col0 + 2 * t + 9) * ld + row0 + g + 8] = __float2bfloat16_rn(v3.y);
}

// acc[m16 x n8] += A(16 rows of AT-transposed data) * B: A(m, k) = AT[m][k] (k = points), B(k, n) = BT[n][k].
FIT_D void mma_from_t(float* acc, const __nv_bfloat16* AT, int m0, const __nv_bfloat16* BT, int n0, int k0, int ld,
                      int lane) {
  const int g = lane >> 2, t = lane & 3;
  uint32_t a[4];
  a[0] = ld32(AT + (m0 + g) * ld + k0 + 2 * t);
  a[1] = ld32(AT + (m0 + g + 8) * ld + k0 + 2 * t);
  a[2] = ld32(AT + (m0 + g) * ld + k0 + 2 * t + 8);
  a[3] = ld32(AT + (m0 + g + 8) * ld + k0 + 2 * t + 8);
  mma_bf16(acc, a, ld32(BT + (n0 + g) * ld + k0 + 2 * t), ld32(BT + (n0 + g) * ld + k0 + 2 * t + 8));
}

__global__ void __launch_bounds__(128) k_mlp_train(const float* __restrict__ Pm, const float* __restrict__ X,
                                                   const float* __restrict__ T, long ld, long P, long Ptot,
                                                   const float* __restrict__ in_scale,
                                                   const float* __restrict__ t_scale, float* __restrict__ grad,
                                                   double* __restrict__ loss, int homog) {
  // weights + staged activations exceed the 48 KB static limit: dynamic shared memory
  extern __shared__ __align__(16) unsigned char mlp_dyn_smem[];
  MlpSmem& w = *reinterpret_cast<MlpSmem*>(mlp_dyn_smem);
  MlpTrainSmem& a = *reinterpret_cast<MlpTrainSmem*>(mlp_dyn_smem + ((sizeof(MlpSmem) + 15) / 16) * 16);
  __shared__ float sc[9], tsc[6], db1[64], db2[64], db3[8];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int g = lane >> 2, t = lane & 3;
  mlp_load_weights(&w, Pm, tid, blockDim.x);
  if (tid < 9) sc[tid] = in_scale[tid];
  if (tid < 6) tsc[tid] = t_scale[tid];
  if (tid < 64) { db1[tid] = 0.f; db2[tid] = 0.f; }
  if (tid < 8) db3[tid] = 0.f;
  __syncthreads();
  // per-warp slices of the weight gradients (FP32 accumulators)
  float gW2[8][4], gW1[2][4], gW3[2][4];
#pragma unroll
  for (int n = 0; n < 8; ++n) gW2[n][0] = gW2[n][1] = gW2[n][2] = gW2[n][3] = 0.f;
#pragma unroll
  for (int n = 0; n < 2; ++n) {
    gW1[n][0] = gW1[n][1] = gW1[n][2] = gW1[n][3] = 0.f;
    gW3[n][0] = gW3[n][1] = gW3[n][2] = gW3[n][3] = 0.f;
  }
  double lsum = 0.0;
  const float inv = 2.f / (float)Ptot;
  const long nblk = (P + 63) / 64;
  for (long blk = blockIdx.x; blk < nblk; blk += gridDim.x) {
    const long p0 = blk * 64 + warp * 16;
    const int r0 = warp * 16;
    uint32_t xa[4], h1a[4][4], h2a[4][4];
    float y[4], sn[2];
    mlp_load_x(X, ld, P, p0, sc, xa, lane, homog != 0, sn);
    mlp_tile_forward(&w, xa, h1a, h2a, y, lane);
    // dY = 2 (s Y - T) s / Ptot on the 6 real outputs (scaled units; s = 1 unless homogeneous)
    float dy[4];
#pragma unroll
    for (int r = 0; r < 2; ++r)
#pragma unroll
      for (int e = 0; e < 2; ++e) {
        const int o = 2 * t + e;
        const long p = p0 + g + 8 * r;
        float d = 0.f;
        if (o < 6 && p < P) {
          const float diff = y[2 * r + e] * sn[r] - T[(long)o * ld + p] * tsc[o];
          lsum += (double)diff * diff;
          d = inv * diff * sn[r];
        }
        dy[2 * r + e] = d;
      }
    // dH2 = (dY W3) * (H2 > 0): A = dY (k = outputs padded to 16), B(k=o, n=h) = W3T[h][o]
    uint32_t dya[4] = {pack_bf16(dy[0], dy[1]), pack_bf16(dy[2], dy[3]), 0u, 0u};
    float dh[8][4];
#pragma unroll
    for (int n = 0; n < 8; ++n) {
      dh[n][0] = dh[n][1] = dh[n][2] = dh[n][3] = 0.f;
      const __nv_bfloat16* br = w.W3T + (n * 8 + g) * 16;
      mma_bf16(dh[n], dya, ld32(br + 2 * t), ld32(br + 2 * t + 8));
    }
    uint32_t dh2a[4][4];
#pragma unroll
    for (int s = 0; s < 4; ++s) {
      const float2 m0 = unpack_bf16(h2a[s][0]), m1 = unpack_bf16(h2a[s][1]);
      const float2 m2 = unpack_bf16(h2a[s][2]), m3 = unpack_bf16(h2a[s][3]);
      const float* lo = dh[2 * s];
      const float* hi = dh[2 * s + 1];
      dh2a[s][0] = pack_bf16(m0.x > 0.f ? lo[0] : 0.f, m0.y > 0.f ? lo[1] : 0.f);
      dh2a[s][1] = pack_bf16(m1.x > 0.f ? lo[2] : 0.f, m1.y > 0.f ? lo[3] : 0.f);
      dh2a[s][2] = pack_bf16(m2.x > 0.f ? hi[0] : 0.f, m2.y > 0.f ? hi[1] : 0.f);
      dh2a[s][3] = pack_bf16(m3.x > 0.f ? hi[2] : 0.f, m3.y > 0.f ? hi[3] : 0.f);
    }
    // dH1 = (dH2 W2) * (H1 > 0): B(k = h2, n = h1) = W2T[h1][h2]
#pragma unroll
    for (int n = 0; n < 8; ++n) {
      dh[n][0] = dh[n][1] = dh[n][2] = dh[n][3] = 0.f;
#pragma unroll
      for (int s = 0; s < 4; ++s) {
        const __nv_bfloat16* br = w.W2T + (n * 8 + g) * 64 + 16 * s;
        mma_bf16(dh[n], dh2a[s], ld32(br + 2 * t), ld32(br + 2 * t + 8));
      }
    }
    uint32_t dh1a[4][4];
#pragma unroll
    for (int s = 0; s < 4; ++s) {
      const float2 m0 = unpack_bf16(h1a[s][0]), m1 = unpack_bf16(h1a[s][1]);
      const float2 m2 = unpack_bf16(h1a[s][2]), m3 = unpack_bf16(h1a[s][3]);
      const float* lo = dh[2 * s];
      const float* hi = dh[2 * s + 1];
      dh1a[s][0] = pack_bf16(m0.x > 0.f ? lo[0] : 0.f, m0.y > 0.f ? lo[1] : 0.f);
      dh1a[s][1] = pack_bf16(m1.x > 0.f ? lo[2] : 0.f, m1.y > 0.f ? lo[3] : 0.f);
      dh1a[s][2] = pack_bf16(m2.x > 0.f ? hi[0] : 0.f, m2.y > 0.f ? hi[1] : 0.f);
      dh1a[s][3] = pack_bf16(m3.x > 0.f ? hi[2] : 0.f, m3.y > 0.f ? hi[3] : 0.f);
    }
    // stage the 64-point block transposed for the weight-gradient reductions
    st_a_transposed(a.XT, 64, 0, r0, xa, lane);
#pragma unroll
    for (int s = 0; s < 4; ++s) {
      st_a_transposed(a.H1T, 64, 16 * s, r0, h1a[s], lane);
      st_a_transposed(a.H2T, 64, 16 * s, r0, h2a[s], lane);
      st_a_transposed(a.dH2T, 64, 16 * s, r0, dh2a[s], lane);
      st_a_transposed(a.dH1T, 64, 16 * s, r0, dh1a[s], lane);
    }
    {
      uint32_t dyfull[4] = {dya[0], dya[1], 0u, 0u};
      st_a_transposed(a.dYT, 64, 0, r0, dyfull, lane);
    }
    __syncthreads();
    // dW2[h2][h1] += sum_p dH2[p][h2] H1[p][h1]: warp w owns rows h2 in [16w, 16w+16)
#pragma unroll
    for (int n = 0; n < 8; ++n)
#pragma unroll
      for (int k0 = 0; k0 < 64; k0 += 16) mma_from_t(gW2[n], a.dH2T, 16 * warp, a.H1T, 8 * n, k0, 64, lane);
    // dW1[h1][f] += sum_p dH1[p][h1] X[p][f]
#pragma unroll
    for (int n = 0; n < 2; ++n)
#pragma unroll
      for (int k0 = 0; k0 < 64; k0 += 16) mma_from_t(gW1[n], a.dH1T, 16 * warp, a.XT, 8 * n, k0, 64, lane);
    // dW3[o][h2] += sum_p dY[p][o] H2[p][h2]: rows o (padded to 16), warp w owns columns [16w, 16w+16)
#pragma unroll
    for (int n = 0; n < 2; ++n)
#pragma unroll
      for (int k0 = 0; k0 < 64; k0 += 16) mma_from_t(gW3[n], a.dYT, 0, a.H2T, 16 * warp + 8 * n, k0, 64, lane);
    // bias gradients: column sums over the block's 64 points
    if (tid < 64) {
      float s1 = 0.f, s2 = 0.f;
      for (int p = 0; p < 64; ++p) {
        s1 += __bfloat162float(a.dH1T[tid * 64 + p]);
        s2 += __bfloat162float(a.dH2T[tid * 64 + p]);
      }
      db1[tid] += s1;
      db2[tid] += s2;
    } else if (tid < 72) {
      float s3 = 0.f;
      for (int p = 0; p < 64; ++p) s3 += __bfloat162float(a.dYT[(tid - 64) * 64 + p]);
      db3[tid - 64] += s3;
    }
    __syncthreads();
  }
  // flush: C fragment element (row, col) of each slice
#pragma unroll
  for (int n = 0; n < 8; ++n)
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      const int row = 16 * warp + g + ((e & 2) ? 8 : 0), col = 8 * n + 2 * t + (e & 1);
      atomicAdd(&grad[MlpOff::W2 + row * 64 + col], gW2[n][e]);
    }
#pragma unroll
  for (int n = 0; n < 2; ++n)
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      const int row = 16 * warp + g + ((e & 2) ? 8 : 0), col = 8 * n + 2 * t + (e & 1);
      atomicAdd(&grad[MlpOff::W1 + row * 16 + col], gW1[n][e]);
      const int orow = g + ((e & 2) ? 8 : 0), hcol = 16 * warp + 8 * n + 2 * t + (e & 1);
      if (orow < 8) atomicAdd(&grad[MlpOff::W3 + orow * 64 + hcol], gW3[n][e]);
    }
  if (tid < 64) {
    atomicAdd(&grad[MlpOff::B1 + tid], db1[tid]);
    atomicAdd(&grad[MlpOff::B2 + tid], db2[tid]);
  }
  if (tid < 8) atomicAdd(&grad[MlpOff::B3 + tid], db3[tid]);
  // loss (sum of squared scaled errors)
  for (int o = 16; o > 0; o >>= 1) lsum += __shfl_down_sync(0xffffffffu, lsum, o);
  if (lane == 0) atomicAdd(loss, lsum);
}

__global__ void k_mlp_adam(float* Pm, const float* __restrict__ gr, float* m, float* v, int n, float lr, float b1,
                           float b2, float eps, float c1, float c2) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float gg = gr[i];
  const float mm = b1 * m[i] + (1.f - b1) * gg;
  const float vv = b2 * v[i] + (1.f - b2) * gg * gg;
  m[i] = mm;
  v[i] = vv;
  Pm[i] -= lr * (mm / c1) / (sqrtf(vv / c2) + eps);
}

// Gradient (Clark) model for a Gaussian filter: tau_ij = ell^2/12 A_ik A_jk; optional tau output,
// Pi = -tau_ij S_ij.
__global__ void k_gradient_model(const float* __restrict__ X, long ld, long P, float c, float* __restrict__ tau,
                                 float* __restrict__ Pi) {
  const long p = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (p >= P) return;
  float A[9];
#pragma unroll
  for (int f = 0; f < 9; ++f) A[f] = X[(long)f * ld + p];
  float pi = 0.f;
#pragma unroll
  for (int o = 0; o < 6; ++o) {
    const int i = o < 3 ? o : (o == 5 ? 1 : 0), j = o < 3 ? o : (o == 3 ? 1 : 2);
    const float t = c * (A[3 * i] * A[3 * j] + A[3 * i + 1] * A[3 * j + 1] + A[3 * i + 2] * A[3 * j + 2]);
    if (tau) tau[(long)o * ld + p] = t;
    pi -= (i == j) ? t * A[3 * i + i] : t * (A[3 * i + j] + A[3 * j + i]);
  }
  if (Pi) Pi[p] = pi;
}

// out = tau - ell^2/12 A A^T: the targets of the network's residual over the gradient model.
__global__ void k_stress_residual(const float* __restrict__ X, const float* __restrict__ tau, long ld, long P, float c,
                                  float* __restrict__ out) {
  const long p = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (p >= P) return;
#pragma unroll
  for (int o = 0; o < 6; ++o) out[(long)o * ld + p] = tau[(long)o * ld + p] - c * gradient_model_stress(o, X, ld, p);
}

// FP64 block sums of nq quantities per thread, one atomicAdd per block and quantity.
template <int NQ>
FIT_D void block_sums_to(double (&q)[NQ], double* out) {
  __shared__ double ws[NQ][32];
#pragma unroll
  for (int k = 0; k < NQ; ++k)
    for (int o = 16; o > 0; o >>= 1) q[k] += __shfl_down_sync(0xffffffffu, q[k], o);
  if ((threadIdx.x & 31) == 0)
#pragma unroll
    for (int k = 0; k < NQ; ++k) ws[k][threadIdx.x >> 5] = q[k];
  __syncthreads();
  if (threadIdx.x < 32) {
#pragma unroll
    for (int k = 0; k < NQ; ++k) {
      double s = threadIdx.x < (blockDim.x >> 5) ? ws[k][threadIdx.x] : 0.0;
      for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
      if (threadIdx.x == 0) atomicAdd(out + k, s);
    }
  }
}

// Per field f < nf: out[2f] += sum x, out[2f+1] += sum x^2.
__global__ void k_moments(const float* __restrict__ X, long ld, long P, int f, double* out) {
  double q[2] = {0.0, 0.0};
  for (long p = blockIdx.x * (long)blockDim.x + threadIdx.x; p < P; p += (long)gridDim.x * blockDim.x) {
    const double v = X[(long)f * ld + p];
    q[0] += v;
    q[1] += v * v;
  }
  block_sums_to<2>(q, out + 2 * f);
}

// out += (sum a, sum b, sum a^2, sum b^2, sum ab, sum (a-b)^2)
__global__ void k_compare(const float* __restrict__ a, const float* __restrict__ b, long P, double* out) {
  double q[6] = {0, 0, 0, 0, 0, 0};
  for (long p = blockIdx.x * (long)blockDim.x + threadIdx.x; p < P; p += (long)gridDim.x * blockDim.x) {
    const double x = a[p], y = b[p];
    q[0] += x;
    q[1] += y;
    q[2] += x * x;
    q[3] += y * y;
    q[4] += x * y;
    q[5] += (x - y) * (x - y);
  }
  block_sums_to<6>(q, out);
}

}  // namespace fit

using namespace fit;

static int* g_mlp_err = nullptr;   // wait-timeout flag of the tcgen05 kernels (read by fit_mlp_status)

static int mlp_err_flag(int** out) {
  if (!g_mlp_err) {
    FIT_CUDA_CHECK(cudaMalloc(&g_mlp_err, sizeof(int)));
    FIT_CUDA_CHECK(cudaMemset(g_mlp_err, 0, sizeof(int)));
  }
  *out = g_mlp_err;
  return FIT_OK;
}

extern "C" int fit_mlp_nparams(void) { return MLP_NPARAM; }

// Reads and clears the tcgen05 forward's wait-timeout flag (synchronises the device): 0 when every
// bounded wait of every earlier forward finished.
extern "C" int fit_mlp_status(int* timed_out) {
  if (!timed_out) {
    fit_set_error("NULL argument");
    return FIT_ERR_ARG;
  }
  *timed_out = 0;
  if (!g_mlp_err) return FIT_OK;
  FIT_CUDA_CHECK(cudaMemcpy(timed_out, g_mlp_err, sizeof(int), cudaMemcpyDeviceToHost));
  FIT_CUDA_CHECK(cudaMemset(g_mlp_err, 0, sizeof(int)));
  return FIT_OK;
}

extern "C" int fit_mlp_forward(const float* params, const float* X, int64_t ld, int64_t P, const float* in_scale,
                               const float* t_scale, int homogeneous, double clark_ell, float* Y, float* Pi,
                               void* stream) {
  if (!params || !X || !in_scale || !t_scale || (!Y && !Pi) || P < 0 || ld < P) {
    fit_set_error("bad argument (need params, X, scales, one of Y/Pi, 0 <= P <= ld)");
    return FIT_ERR_ARG;
  }
  if (P == 0) return FIT_OK;
  cudaStream_t st = (cudaStream_t)stream;
  const char* env = getenv("FIT_MLP_MMASYNC");   // the mma.sync forward (kept for comparison)
  if (env && env[0] == '1') {
    const long ntile = (P + 15) / 16;
    long blocks = (ntile + 7) / 8;
    if (blocks > 152 * 8) blocks = 152 * 8;
    k_mlp_forward<<<(unsigned)blocks, 256, 0, st>>>(params, X, ld, P, in_scale, t_scale, Y, Pi, homogeneous,
                                                     (float)(clark_ell * clark_ell / 12.0));
    FIT_LAUNCH_CHECK();
    return FIT_OK;
  }
  int* err = nullptr;
  FIT_TRY(mlp_err_flag(&err));
  static int nsm = 0;
  if (!nsm) {
    int dev = 0;
    FIT_CUDA_CHECK(cudaGetDevice(&dev));
    FIT_CUDA_CHECK(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
    FIT_CUDA_CHECK(cudaFuncSetAttribute(k_mlp_forward_tc, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        (int)sizeof(MlpTcSmem)));
  }
  const long ntile = (P + 127) / 128;
  long blocks = (long)nsm * 6;   // six CTAs per SM: 6 x 64 tensor-memory columns, ~6 x 34 KB shared memory
  if (blocks > ntile) blocks = ntile;
  k_mlp_forward_tc<<<(unsigned)blocks, 128, sizeof(MlpTcSmem), st>>>(params, X, ld, P, in_scale, t_scale, Y, Pi,
                                                                    homogeneous,
                                                                    (float)(clark_ell * clark_ell / 12.0), err,
                                                                    fit_wait_cycles());
  FIT_LAUNCH_CHECK();
  return FIT_OK;
}

extern "C" int fit_mlp_train_grad(const float* params, const float* X, const float* T, int64_t ld, int64_t P,
                                  int64_t Ptot, const float* in_scale, const float* t_scale, int homogeneous,
                                  float* grad, double* loss, void* stream) {
  if (!params || !X || !T || !in_scale || !t_scale || !grad || !loss || P <= 0 || Ptot <= 0 || ld < P) {
    fit_set_error("bad argument");
    return FIT_ERR_ARG;
  }
  cudaStream_t st = (cudaStream_t)stream;
  const char* env = getenv("FIT_MLP_MMASYNC");   // the mma.sync training step (kept for comparison)
  if (!(env && env[0] == '1')) {
    int* err = nullptr;
    FIT_TRY(mlp_err_flag(&err));
    static bool tc_attr = false;
    if (!tc_attr) {
      FIT_CUDA_CHECK(cudaFuncSetAttribute(k_mlp_train_tc, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          (int)sizeof(MlpTrainTcSmem)));
      tc_attr = true;
    }
    int dev = 0, nsm = 0;
    FIT_CUDA_CHECK(cudaGetDevice(&dev));
    FIT_CUDA_CHECK(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
    const long ntile = (P + 127) / 128;
    const long blocks = ntile < nsm ? ntile : nsm;   // one CTA per SM (256 tensor-memory columns, ~117 KB)
    k_mlp_train_tc<<<(unsigned)blocks, 128, sizeof(MlpTrainTcSmem), st>>>(params, X, T, ld, P, Ptot, in_scale,
                                                                           t_scale, grad, loss, homogeneous, err,
                                                                           fit_wait_cycles());
    FIT_LAUNCH_CHECK();
    return FIT_OK;
  }
  const long nblk = (P + 63) / 64;
  long blocks = nblk < 152 * 4 ? nblk : 152 * 4;
  const size_t smem = ((sizeof(MlpSmem) + 15) / 16) * 16 + sizeof(MlpTrainSmem);
  static bool attr_set[64] = {};
  int dev = 0;
  FIT_CUDA_CHECK(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64 || !attr_set[dev]) {
    FIT_CUDA_CHECK(cudaFuncSetAttribute(k_mlp_train, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    if (dev >= 0 && dev < 64) attr_set[dev] = true;
  }
  k_mlp_train<<<(unsigned)blocks, 128, smem, st>>>(params, X, T, ld, P, Ptot, in_scale, t_scale, grad, loss,
                                                    homogeneous);
  FIT_LAUNCH_CHECK();
  return FIT_OK;
}

extern "C" int fit_mlp_adam(float* params, const float* grad, float* m, float* v, int step, float lr, float beta1,
                            float beta2, float eps, void* stream) {
  if (!params || !grad || !m || !v || step < 1) {
    fit_set_error("bad argument");
    return FIT_ERR_ARG;
  }
  const float c1 = 1.f - powf(beta1, (float)step), c2 = 1.f - powf(beta2, (float)step);
  k_mlp_adam<<<(MLP_NPARAM + 255) / 256, 256, 0, (cudaStream_t)stream>>>(params, grad, m, v, MLP_NPARAM, lr, beta1,
                                                                        beta2, eps, c1, c2);
  FIT_LAUNCH_CHECK();
  return FIT_OK;
}

extern "C" int fit_gradient_model_flux(const float* A, int64_t ld, int64_t P, double ell, float* tau, float* Pi,
                                       void* stream) {
  if (!A || (!tau && !Pi) || P < 0 || ld < P || !(ell > 0.0)) {
    fit_set_error("bad argument (need A, one of tau/Pi, 0 <= P <= ld, ell > 0)");
    return FIT_ERR_ARG;
  }
  if (P == 0) return FIT_OK;
  k_gradient_model<<<(unsigned)((P + 255) / 256), 256, 0, (cudaStream_t)stream>>>(A, ld, P, (float)(ell * ell / 12.0),
                                                                                  tau, Pi);
  FIT_LAUNCH_CHECK();
  return FIT_OK;
}

extern "C" int fit_field_moments(const float* X, int64_t ld, int64_t P, int nf, double* out, void* stream) {
  if (!X || !out || P <= 0 || ld < P || nf <= 0) {
    fit_set_error("bad argument");
    return FIT_ERR_ARG;
  }
  cudaStream_t st = (cudaStream_t)stream;
  FIT_CUDA_CHECK(cudaMemsetAsync(out, 0, sizeof(double) * 2 * nf, st));
  long blocks = (P + 255) / 256;
  if (blocks > 152 * 8) blocks = 152 * 8;
  for (int f = 0; f < nf; ++f) {
    k_moments<<<(unsigned)blocks, 256, 0, st>>>(X, ld, P, f, out);
    FIT_LAUNCH_CHECK();
  }
  return FIT_OK;
}

extern "C" int fit_field_compare(const float* a, const float* b, int64_t P, double* out, void* stream) {
  if (!a || !b || !out || P <= 0) {
    fit_set_error("bad argument");
    return FIT_ERR_ARG;
  }
  cudaStream_t st = (cudaStream_t)stream;
  FIT_CUDA_CHECK(cudaMemsetAsync(out, 0, sizeof(double) * 6, st));
  long blocks = (P + 255) / 256;
  if (blocks > 152 * 8) blocks = 152 * 8;
  k_compare<<<(unsigned)blocks, 256, 0, st>>>(a, b, P, out);
  FIT_LAUNCH_CHECK();
  return FIT_OK;
}

extern "C" int fit_stress_residual(const float* A, const float* tau, int64_t ld, int64_t P, double ell, float* out,
                                   void* stream) {
  if (!A || !tau || !out || P < 0 || ld < P || !(ell > 0.0)) {
    fit_set_error("bad argument (need A, tau, out, 0 <= P <= ld, ell > 0)");
    return FIT_ERR_ARG;
  }
  if (P == 0) return FIT_OK;
  k_stress_residual<<<(unsigned)((P + 255) / 256), 256, 0, (cudaStream_t)stream>>>(A, tau, ld, P,
                                                                                  (float)(ell * ell / 12.0), out);
  FIT_LAUNCH_CHECK();
  return FIT_OK;
}
