// Fused shell-to-shell kernels instantiated for cube sizes 96 192 384 768.
#include "fit_fused_impl.cuh"

namespace fit {

// Returns 1 when N is not built in this translation unit.
int fz_dispatch_b(int N, const FzArgs& a, const float2* H, const float2* Ceff, const uint16_t* seff,
                    const float* kd, const float* U, float2* bufA, float2* bufB,
                    double* partial, const float2* tw, int* err, cudaStream_t st) {
  switch (N) {
    case 96: return fz_batch<96>(a, H, Ceff, seff, kd, U, bufA, bufB, partial, tw, err, st);
    case 192: return fz_batch<192>(a, H, Ceff, seff, kd, U, bufA, bufB, partial, tw, err, st);
    case 384: return fz_batch<384>(a, H, Ceff, seff, kd, U, bufA, bufB, partial, tw, err, st);
    case 768: return fz_batch<768>(a, H, Ceff, seff, kd, U, bufA, bufB, partial, tw, err, st);
    default: return 1;
  }
}

// zinv of a batch over pencil tiles [t0, t1) (1 when N is not built here).
int fz_zinv_b(int N, const FzArgs& a, const float2* H, const float* kd, float2* bufA, const float2* tw, int t0,
               int t1, cudaStream_t st) {
  switch (N) {
    case 96: return fz_zinv_tiles<96>(a, H, kd, bufA, tw, t0, t1, st);
    case 192: return fz_zinv_tiles<192>(a, H, kd, bufA, tw, t0, t1, st);
    case 384: return fz_zinv_tiles<384>(a, H, kd, bufA, tw, t0, t1, st);
    case 768: return fz_zinv_tiles<768>(a, H, kd, bufA, tw, t0, t1, st);
    default: return 1;
  }
}

// Pencils per tile of the fused strided passes for transform length N (0 when not built here).
int fz_tile_cols_b(int N) {
  switch (N) {
    case 96: return FzTile<96>::C;
    case 192: return FzTile<192>::C;
    case 384: return FzTile<384>::C;
    case 768: return FzTile<768>::C;
    default: return 0;
  }
}

// Self-advecting velocity in physical space over the live box (1 when N is not built here).
int fz_velocity_b(int N, const FzArgs& a, const float2* H, float2* bufZ, float2* bufY, float* U, const float2* tw,
                   float scale, cudaStream_t st) {
  switch (N) {
    case 96: return fz_velocity<96>(a, H, bufZ, bufY, U, tw, scale, st);
    case 192: return fz_velocity<192>(a, H, bufZ, bufY, U, tw, scale, st);
    case 384: return fz_velocity<384>(a, H, bufZ, bufY, U, tw, scale, st);
    case 768: return fz_velocity<768>(a, H, bufZ, bufY, U, tw, scale, st);
    default: return 1;
  }
}

// Whole-box nonlinear terms of a batch (1 when N is not built here).
int fz_terms_b(int N, const FzArgs& a, const float2* H, const float* kd, const float* U, float2* bufA, float2* bufB,
               float2* Nout, const float2* tw, int* err, cudaStream_t st) {
  switch (N) {
    case 96: return fz_terms<96>(a, H, kd, U, bufA, bufB, Nout, tw, err, st);
    case 192: return fz_terms<192>(a, H, kd, U, bufA, bufB, Nout, tw, err, st);
    case 384: return fz_terms<384>(a, H, kd, U, bufA, bufB, Nout, tw, err, st);
    case 768: return fz_terms<768>(a, H, kd, U, bufA, bufB, Nout, tw, err, st);
    default: return 1;
  }
}

}  // namespace fit
