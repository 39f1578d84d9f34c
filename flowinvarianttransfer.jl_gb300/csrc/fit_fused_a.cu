// Fused shell-to-shell kernels instantiated for cube sizes 64 128 256 512.
#include "fit_fused_impl.cuh"

namespace fit {

// Returns 1 when N is not built in this translation unit.
int fz_dispatch_a(int N, const FzArgs& a, const float2* H, const float2* Ceff, const uint16_t* seff,
                    const float* kd, const float* U, float2* bufA, float2* bufB,
                    double* partial, const float2* tw, int* err, cudaStream_t st) {
  switch (N) {
    case 64: return fz_batch<64>(a, H, Ceff, seff, kd, U, bufA, bufB, partial, tw, err, st);
    case 128: return fz_batch<128>(a, H, Ceff, seff, kd, U, bufA, bufB, partial, tw, err, st);
    case 256: return fz_batch<256>(a, H, Ceff, seff, kd, U, bufA, bufB, partial, tw, err, st);
    case 512: return fz_batch<512>(a, H, Ceff, seff, kd, U, bufA, bufB, partial, tw, err, st);
    default: return 1;
  }
}

// Pencils per tile of the fused strided passes for transform length N (0 when not built here).
int fz_tile_cols_a(int N) {
  switch (N) {
    case 64: return FzTile<64>::C;
    case 128: return FzTile<128>::C;
    case 256: return FzTile<256>::C;
    case 512: return FzTile<512>::C;
    default: return 0;
  }
}

// Self-advecting velocity in physical space over the live box (1 when N is not built here).
int fz_velocity_a(int N, const FzArgs& a, const float2* H, float2* bufZ, float2* bufY, float* U, const float2* tw,
                   float scale, cudaStream_t st) {
  switch (N) {
    case 64: return fz_velocity<64>(a, H, bufZ, bufY, U, tw, scale, st);
    case 128: return fz_velocity<128>(a, H, bufZ, bufY, U, tw, scale, st);
    case 256: return fz_velocity<256>(a, H, bufZ, bufY, U, tw, scale, st);
    case 512: return fz_velocity<512>(a, H, bufZ, bufY, U, tw, scale, st);
    default: return 1;
  }
}

// Whole-box nonlinear terms of a batch (1 when N is not built here).
int fz_terms_a(int N, const FzArgs& a, const float2* H, const float* kd, const float* U, float2* bufA, float2* bufB,
               float2* Nout, const float2* tw, int* err, cudaStream_t st) {
  switch (N) {
    case 64: return fz_terms<64>(a, H, kd, U, bufA, bufB, Nout, tw, err, st);
    case 128: return fz_terms<128>(a, H, kd, U, bufA, bufB, Nout, tw, err, st);
    case 256: return fz_terms<256>(a, H, kd, U, bufA, bufB, Nout, tw, err, st);
    case 512: return fz_terms<512>(a, H, kd, U, bufA, bufB, Nout, tw, err, st);
    default: return 1;
  }
}

}  // namespace fit
