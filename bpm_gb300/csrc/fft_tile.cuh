// Shared-memory tile FFT: 16 independent complex sequences of length N, transformed
// together by one thread block. This is the building block of every FFT pass of the
// split-step march (row passes along x, column passes along y).
//
// Layout. Element n of sequence c (c = 0..15) lives at tile[n*16 + (c ^ (n & 15))].
// Every FFT stage maps the 16 threads of a half-warp onto the 16 sequences at the same
// n, so each half-warp touches one 128-byte row of the tile: all shared-memory accesses
// of the butterfly stages are free of bank conflicts whatever the stage stride. The XOR
// swizzle keeps the transposing loads of row tiles (one sequence = one image row) to at
// most 4-way conflicts instead of 32-way.
//
// Algorithm. Stockham autosort, radix RS per stage, natural order in and out (Govindaraju
// et al., "High performance discrete Fourier transforms on graphics processors", SC'08):
// for Ns = 1, RS0, RS0*RS1, ... each butterfly j reads x[j + r*N/RS], multiplies by
// W_N^{(j mod Ns)*r*N/(Ns*RS)}, does a radix-RS DFT in registers and writes to
// (j/Ns)*Ns*RS + (j mod Ns) + r*Ns. Every thread holds R values (R >= RS) and runs R/RS
// butterflies per stage; a stage reads into registers, synchronises and writes back in
// place, so the tile needs no second buffer. Twiddles come from a per-size table
// W_N^k = exp(-2 pi i k / N) computed in FP64 on the host.
//
// Sign convention: forward = exp(-i...), unnormalised; inverse = exp(+i...), unnormalised.
#pragma once

#include "common.cuh"

namespace bpmgb {

__device__ __forceinline__ int tile_idx(int n, int c) { return (n << 4) + (c ^ (n & 15)); }

// multiply by -i (forward) or +i (inverse)
template <bool INV>
__device__ __forceinline__ float2 mul_mi(float2 a) {
  return INV ? make_float2(-a.y, a.x) : make_float2(a.y, -a.x);
}

template <int R, bool INV>
struct Dft;

template <bool INV>
struct Dft<2, INV> {
  __device__ __forceinline__ static void run(float2* v) {
    float2 a = v[0], b = v[1];
    v[0] = cadd(a, b);
    v[1] = csub(a, b);
  }
};

template <bool INV>
struct Dft<4, INV> {
  __device__ __forceinline__ static void run(float2* v) {
    float2 a0 = cadd(v[0], v[2]);
    float2 a1 = csub(v[0], v[2]);
    float2 a2 = cadd(v[1], v[3]);
    float2 a3 = mul_mi<INV>(csub(v[1], v[3]));
    v[0] = cadd(a0, a2);
    v[2] = csub(a0, a2);
    v[1] = cadd(a1, a3);
    v[3] = csub(a1, a3);
  }
};

// radix-8 and radix-16 by one even/odd split into two half-size DFTs
template <bool INV>
struct Dft<8, INV> {
  __device__ __forceinline__ static void run(float2* v) {
    constexpr float c = 0.70710678118654752f;
    float2 e[4] = {v[0], v[2], v[4], v[6]};
    float2 o[4] = {v[1], v[3], v[5], v[7]};
    Dft<4, INV>::run(e);
    Dft<4, INV>::run(o);
    const float s = INV ? 1.f : -1.f;  // sign of the imaginary part of W8^1
    float2 t1 = make_float2(c * (o[1].x - s * o[1].y), c * (o[1].y + s * o[1].x));
    float2 t2 = mul_mi<INV>(o[2]);
    float2 t3 = make_float2(-c * (o[3].x + s * o[3].y), c * (s * o[3].x - o[3].y));
    v[0] = cadd(e[0], o[0]);
    v[4] = csub(e[0], o[0]);
    v[1] = cadd(e[1], t1);
    v[5] = csub(e[1], t1);
    v[2] = cadd(e[2], t2);
    v[6] = csub(e[2], t2);
    v[3] = cadd(e[3], t3);
    v[7] = csub(e[3], t3);
  }
};

template <bool INV>
struct Dft<16, INV> {
  __device__ __forceinline__ static void run(float2* v) {
    float2 e[8], o[8];
#pragma unroll
    for (int i = 0; i < 8; i++) {
      e[i] = v[2 * i];
      o[i] = v[2 * i + 1];
    }
    Dft<8, INV>::run(e);
    Dft<8, INV>::run(o);
    // W16^k = cos(2 pi k/16) -/+ i sin(2 pi k/16), k = 0..7
    constexpr float C[8] = {1.f, 0.92387953251128674f, 0.70710678118654752f, 0.38268343236508977f,
                            0.f, -0.38268343236508977f, -0.70710678118654752f, -0.92387953251128674f};
    constexpr float S[8] = {0.f, 0.38268343236508977f, 0.70710678118654752f, 0.92387953251128674f,
                            1.f, 0.92387953251128674f, 0.70710678118654752f, 0.38268343236508977f};
#pragma unroll
    for (int k = 0; k < 8; k++) {
      float2 w = make_float2(C[k], INV ? S[k] : -S[k]);
      float2 t = (k == 0) ? o[0] : (k == 4 ? mul_mi<INV>(o[4]) : cmul(o[k], w));
      v[k] = cadd(e[k], t);
      v[k + 8] = csub(e[k], t);
    }
  }
};

// radix-32 by one even/odd split into two 16-point DFTs: X[k] = E[k] + W32^k O[k],
// X[k+16] = E[k] - W32^k O[k]
template <bool INV>
struct Dft<32, INV> {
  __device__ __forceinline__ static void run(float2* v) {
    float2 e[16], o[16];
#pragma unroll
    for (int i = 0; i < 16; i++) {
      e[i] = v[2 * i];
      o[i] = v[2 * i + 1];
    }
    Dft<16, INV>::run(e);
    Dft<16, INV>::run(o);
    // W32^k = cos(2 pi k/32) -/+ i sin(2 pi k/32), k = 0..15
    constexpr float C[16] = {1.f, 0.98078528040323044913f, 0.92387953251128675613f, 0.83146961230254523708f,
                             0.70710678118654752440f, 0.55557023301960222474f, 0.38268343236508977173f,
                             0.19509032201612826785f, 0.f, -0.19509032201612826785f, -0.38268343236508977173f,
                             -0.55557023301960222474f, -0.70710678118654752440f, -0.83146961230254523708f,
                             -0.92387953251128675613f, -0.98078528040323044913f};
    constexpr float S[16] = {0.f, 0.19509032201612826785f, 0.38268343236508977173f, 0.55557023301960222474f,
                             0.70710678118654752440f, 0.83146961230254523708f, 0.92387953251128675613f,
                             0.98078528040323044913f, 1.f, 0.98078528040323044913f, 0.92387953251128675613f,
                             0.83146961230254523708f, 0.70710678118654752440f, 0.55557023301960222474f,
                             0.38268343236508977173f, 0.19509032201612826785f};
#pragma unroll
    for (int k = 0; k < 16; k++) {
      const float2 w = make_float2(C[k], INV ? S[k] : -S[k]);
      const float2 t = (k == 0) ? o[0] : (k == 8 ? mul_mi<INV>(o[8]) : cmul(o[k], w));
      v[k] = cadd(e[k], t);
      v[k + 16] = csub(e[k], t);
    }
  }
};

// One Stockham stage of radix RS with stride NS over the 16-sequence tile.
// Thread (c, jt): c = sequence, jt = 0 .. N/R-1.
template <int N, int R, int RS, int NS, bool INV>
__device__ __forceinline__ void tile_stage(float2* tile, const float2* __restrict__ tw, int c, int jt) {
  constexpr int Q = R / RS;           // butterflies per thread
  constexpr int STRIDE_IN = N / RS;
  constexpr int TWSTEP = N / (NS * RS);
  float2 v[R];
#pragma unroll
  for (int q = 0; q < Q; q++) {
    const int j = jt * Q + q;
#pragma unroll
    for (int r = 0; r < RS; r++) v[q * RS + r] = tile[tile_idx(j + r * STRIDE_IN, c)];
  }
#pragma unroll
  for (int q = 0; q < Q; q++) {
    const int j = jt * Q + q;
    if (NS > 1) {
      const int jm = j & (NS - 1);
#pragma unroll
      for (int r = 1; r < RS; r++) {
        float2 w = tw[jm * r * TWSTEP];
        if (INV) w.y = -w.y;
        v[q * RS + r] = cmul(v[q * RS + r], w);
      }
    }
    Dft<RS, INV>::run(&v[q * RS]);
  }
  __syncthreads();
#pragma unroll
  for (int q = 0; q < Q; q++) {
    const int j = jt * Q + q;
    const int jm = j & (NS - 1);
    const int base = (j / NS) * NS * RS + jm;
#pragma unroll
    for (int r = 0; r < RS; r++) tile[tile_idx(base + r * NS, c)] = v[q * RS + r];
  }
  __syncthreads();
}

template <int N, int R, int NS, bool INV>
__device__ __forceinline__ void tile_fft_from(float2* tile, const float2* __restrict__ tw, int c, int jt) {
  if constexpr (NS < N) {
    constexpr int REM = N / NS;
    constexpr int RS = REM < R ? REM : R;
    tile_stage<N, R, RS, NS, INV>(tile, tw, c, jt);
    tile_fft_from<N, R, NS * RS, INV>(tile, tw, c, jt);
  }
}

// Full length-N FFT of the 16 sequences of `tile`. Needs 16*N/R threads; callers with
// more threads leave the surplus idle (they must still reach every __syncthreads).
template <int N, int R, bool INV>
__device__ __forceinline__ void tile_fft(float2* tile, const float2* __restrict__ tw) {
  const int t = threadIdx.x;
  const int c = t & 15;
  const int jt = t >> 4;
  tile_fft_from<N, R, 1, INV>(tile, tw, c, jt);
}

// Thread radix per length: 8 up to 256 points, 16 beyond.
template <int N>
struct TileCfg {
  static constexpr int R = (N <= 8) ? N : (N <= 256 ? 8 : 16);
  static constexpr int THREADS = 16 * N / R;
  static constexpr size_t SMEM = (size_t)N * 16 * sizeof(float2) + (size_t)N * sizeof(float2);
  // blocks per SM the register budget must allow: 2048 threads per SM, i.e. 64 registers
  static constexpr int MINB = THREADS >= 1024 ? 1 : 1024 / THREADS;
};

}  // namespace bpmgb
