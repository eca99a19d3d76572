// Warp-level FFT: L lanes (a warp, L = 32, or a half-warp, L = 16) transform one complex
// sequence of length N (64 <= N <= 1024) held in registers, E = N/L values per lane (16
// for N = 512 on a warp, 32 for N = 1024 on a warp or N = 512 on a half-warp).
//
// Distribution. On entry and on exit lane t holds elements t + L*m, m = 0 .. E-1, in v[m]:
// natural order, consecutive elements on consecutive lanes. So a row of an image is loaded
// and stored with fully coalesced accesses, and the output of an inverse transform is
// already laid out as the input of the next forward transform (no exchange between them).
//
// Algorithm. Stockham autosort (the same radix recurrence as fft_tile.cuh): stages of
// radix RS <= E with stride NS = 1, RS0, RS0*RS1, ...; butterfly j = L*q + t of a stage
// reads x[j + r*N/RS], applies W_N^{(j mod NS)*r*N/(NS*RS)}, runs a radix-RS DFT in
// registers and writes (j/NS)*NS*RS + (j mod NS) + r*NS. The first stage reads its inputs
// from the lane's own registers and the last stage writes its outputs back to them (both
// fall on the lane's t + L*m elements); the stages in between exchange through a private
// per-sequence shared-memory buffer synchronised with __syncwarp over the sequence's lanes,
// with one pad element every 2^S (index p + p >> S; S = 5 when lanes write runs of E = 32,
// else 4), which keeps every exchange at the minimum number of shared-memory wavefronts.
// Fewer lanes with more values each mean fewer stages: 512 points take three stages (two
// exchanges) on a warp, two (one exchange) on a half-warp.
#pragma once

#include "fft_tile.cuh"

namespace bpmgb {

__host__ __device__ constexpr int pad_shift(int N, int L = 32) { return N / L >= 32 ? 5 : 4; }

// Twiddles are stored per stage, entry (r-1)*NS + jm of stage (RS, NS) holding
// W_N^{jm*r*N/(NS*RS)} for r = 1..RS-1, jm = 0..NS-1, stages in march order, stages with
// NS = 1 (no twiddles) skipped. A stage's lanes then read consecutive entries.
__host__ __device__ constexpr int wtw_offset(int N, int ns_target, int L = 32) {
  int off = 0, ns = 1;
  const int E = N / L;
  while (ns < ns_target) {
    const int rs = (N / ns) < E ? (N / ns) : E;
    if (ns > 1) off += (rs - 1) * ns;
    ns *= rs;
  }
  return off;
}
__host__ __device__ constexpr int wtw_size(int N, int L = 32) { return wtw_offset(N, N, L); }

template <int N, int L = 32>
struct WarpFft {
  static constexpr int E = N / L;                          // values per lane
  static constexpr int BUF = N + (N >> pad_shift(N, L));  // padded exchange buffer (float2)
  static constexpr int TW = wtw_size(N, L);                // stage-ordered twiddle entries
};

// lanes of the calling thread's sequence, for __syncwarp
template <int L>
__device__ __forceinline__ unsigned seq_mask() {
  return L == 32 ? 0xffffffffu : (((1u << L) - 1u) << (threadIdx.x & (32 - L)));
}

// Exchange-buffer addressing. Every index a stage touches splits exactly into a per-lane
// part (computed once) and a compile-time offset, so each shared-memory access is one
// instruction with an immediate offset instead of recomputing p + (p >> S) per access.
//   loads:  wpad(q*L + t + r*(N/RS))              = (t + t>>S) + wpad(q*L + r*N/RS)
//   stores: wpad((j/NS)*NS*RS + j%NS + r*NS), j = q*L + t
//           NS >= L: (t + t>>S) + wpad((q*L/NS)*NS*RS + (q*L)%NS + r*NS)
//           NS <  L: B + (((t/NS)*NS*RS) >> S) + wpad(q*L*RS) + r*NS + ((r*NS) >> S),
//                     B = (t/NS)*NS*RS + t%NS
// (warp_index_check verifies both against the direct formula for every lane at compile time.)
__host__ __device__ constexpr int wpad_c(int N, int p, int L = 32) { return p + (p >> pad_shift(N, L)); }
__host__ __device__ constexpr int ld_lane(int N, int L, int t) { return t + (t >> pad_shift(N, L)); }
__host__ __device__ constexpr int ld_off(int N, int L, int RS, int q, int r) {
  return wpad_c(N, q * L + r * (N / RS), L);
}
__host__ __device__ constexpr int st_lane(int N, int L, int RS, int NS, int t) {
  return NS >= L ? t + (t >> pad_shift(N, L))
                 : (t / NS) * NS * RS + t % NS + (((t / NS) * NS * RS) >> pad_shift(N, L));
}
__host__ __device__ constexpr int st_off(int N, int L, int RS, int NS, int q, int r) {
  return NS >= L ? wpad_c(N, (q * L / NS) * NS * RS + (q * L) % NS + r * NS, L)
                 : wpad_c(N, q * L * RS, L) + r * NS + ((r * NS) >> pad_shift(N, L));
}
__host__ __device__ constexpr bool warp_index_check(int N, int L, int RS, int NS) {
  const int Q = (N / L) / RS;
  for (int t = 0; t < L; t++)
    for (int q = 0; q < Q; q++)
      for (int r = 0; r < RS; r++) {
        if (ld_lane(N, L, t) + ld_off(N, L, RS, q, r) != wpad_c(N, q * L + t + r * (N / RS), L)) return false;
        const int j = q * L + t;
        if (st_lane(N, L, RS, NS, t) + st_off(N, L, RS, NS, q, r) !=
            wpad_c(N, (j / NS) * NS * RS + j % NS + r * NS, L))
          return false;
      }
  return true;
}

template <int N, int RS, int NS, bool INV, bool FIRST, bool LAST, int L = 32>
__device__ __forceinline__ void warp_stage(float2 (&v)[N / L], float2* buf, const float2* __restrict__ tw,
                                           int t) {
  constexpr int E = N / L;
  constexpr int Q = E / RS;                    // butterflies per lane
  constexpr int TWOFF = wtw_offset(N, NS, L);  // this stage's twiddle block
  static_assert(warp_index_check(N, L, RS, NS), "exchange-buffer index split");
  float2 a[E];
  if constexpr (FIRST) {
#pragma unroll
    for (int q = 0; q < Q; q++)
#pragma unroll
      for (int r = 0; r < RS; r++) a[q * RS + r] = v[q + r * Q];
  } else {
    const float2* bl = buf + ld_lane(N, L, t);
#pragma unroll
    for (int q = 0; q < Q; q++)
#pragma unroll
      for (int r = 0; r < RS; r++) a[q * RS + r] = bl[ld_off(N, L, RS, q, r)];
  }
  if constexpr (NS > 1) {
    // twiddle W^{(j mod NS) r N/(NS RS)} for j = q*L + t: entry (r-1)*NS + jm of the stage
    const float2* twl = tw + TWOFF + (NS >= L ? t : (t & (NS - 1)));
#pragma unroll
    for (int q = 0; q < Q; q++)
#pragma unroll
      for (int r = 1; r < RS; r++) {
        float2 w = twl[(r - 1) * NS + (NS >= L ? (q * L) % NS : 0)];
        if (INV) w.y = -w.y;
        a[q * RS + r] = cmul(a[q * RS + r], w);
      }
  }
#pragma unroll
  for (int q = 0; q < Q; q++) Dft<RS, INV>::run(&a[q * RS]);
  if constexpr (LAST) {
#pragma unroll
    for (int q = 0; q < Q; q++)
#pragma unroll
      for (int r = 0; r < RS; r++) v[q + r * (NS / L)] = a[q * RS + r];
  } else {
    const unsigned m = seq_mask<L>();
    __syncwarp(m);  // every lane is done reading the buffer (previous stage or transform)
    float2* bs = buf + st_lane(N, L, RS, NS, t);
#pragma unroll
    for (int q = 0; q < Q; q++)
#pragma unroll
      for (int r = 0; r < RS; r++) bs[st_off(N, L, RS, NS, q, r)] = a[q * RS + r];
    __syncwarp(m);
  }
}

template <int N, int NS, bool INV, int L>
__device__ __forceinline__ void warp_fft_from(float2 (&v)[N / L], float2* buf, const float2* __restrict__ tw,
                                              int t) {
  if constexpr (NS < N) {
    constexpr int E = N / L;
    constexpr int REM = N / NS;
    constexpr int RS = REM < E ? REM : E;
    warp_stage<N, RS, NS, INV, NS == 1, NS * RS == N, L>(v, buf, tw, t);
    warp_fft_from<N, NS * RS, INV, L>(v, buf, tw, t);
  }
}

// In-place length-N FFT of the sequence v of L lanes (forward: exp(-i..), inverse:
// exp(+i..), both unnormalised); t = lane within the sequence (0..L-1). buf:
// WarpFft<N, L>::BUF float2 of shared memory private to the sequence; tw: the stage-ordered
// twiddle table (WarpFft<N, L>::TW entries, see wtw_offset).
template <int N, bool INV, int L = 32>
__device__ __forceinline__ void warp_fft(float2 (&v)[N / L], float2* buf, const float2* __restrict__ tw, int t) {
  static_assert(N >= 64 && N <= 1024 && (L == 32 || L == 16), "warp FFT covers 64..1024 points");
  warp_fft_from<N, 1, INV, L>(v, buf, tw, t);
}

// ---- column-split transform ------------------------------------------------------------
// A block holding C length-N columns in the coalesced tile mapping with L threads per
// column — thread (r0, cc) = (tid / C, tid % C) holds rows r0 + L i, i = 0 .. E-1, of column
// cc — can run the first and the last Stockham stage without an exchange: the first stage's
// butterfly j = r0 reads rows r0 + L r, and the last stage (stride NS_LAST >= L, radix
// N/NS_LAST) has butterflies j = r0 + L q writing rows j + NS_LAST r, which are rows r0 + L i
// again. Only the middle stages run per sequence (the L threads tid / L == w on column w)
// through the column's exchange buffer. Butterflies, twiddle entries and operation order
// are warp_fft's, so a column gets the same bits as from warp_fft<N, INV, L>, while the tile
// transposition through shared memory (a store and a load per element on each side of the
// transform) disappears.
__host__ __device__ constexpr int colsplit_last_ns(int N, int L = 32) {
  int ns = 1;
  const int E = N / L;
  while (true) {
    const int rs = (N / ns) < E ? (N / ns) : E;
    if (ns * rs == N) return ns;
    ns *= rs;
  }
}

template <int N, int L = 32>
struct ColSplit {
  static constexpr int E = N / L;
  static constexpr int NS_LAST = colsplit_last_ns(N, L);
  static_assert(NS_LAST >= L && NS_LAST < N, "last stage spans whole L-row groups");
};

// padded positions the tile-mapping stages use, split as in colsplit_first / colsplit_last
// (checked against the direct formula for every thread at compile time)
__host__ __device__ constexpr bool colsplit_index_check(int N, int L) {
  const int E = N / L, S = pad_shift(N, L), NS = colsplit_last_ns(N, L), RS = N / NS;
  for (int r0 = 0; r0 < L; r0++) {
    for (int r = 0; r < E; r++)
      if (r0 * E + ((r0 * E) >> S) + r != wpad_c(N, r0 * E + r, L)) return false;
    for (int q = 0; q < NS / L; q++)
      for (int r = 0; r < RS; r++)
        if (r0 + (r0 >> S) + L * q + ((L * q) >> S) + (NS + (NS >> S)) * r != wpad_c(N, r0 + L * q + NS * r, L))
          return false;
  }
  return true;
}

// first stage (radix E, stride 1) of column cc from the thread's rows r0 + L r, written to
// positions r0*E + r of the column's buffer (padded index p + (p >> S); r0*E + r stays
// inside one 2^S-element run, so the pad is that of r0*E)
template <int N, bool INV, int L = 32>
__device__ __forceinline__ void colsplit_first(const float2 (&v)[N / L], float2* colbuf, int r0) {
  constexpr int E = N / L;
  static_assert(colsplit_index_check(N, L), "column-split index split");
  float2 a[E];
#pragma unroll
  for (int r = 0; r < E; r++) a[r] = v[r];
  Dft<E, INV>::run(a);
  float2* b = colbuf + r0 * E + ((r0 * E) >> pad_shift(N, L));
#pragma unroll
  for (int r = 0; r < E; r++) b[r] = a[r];
}

// middle stages (stride E .. NS_LAST), per sequence on its own column buffer; the caller
// makes the first stage's stores visible before and synchronises the block after
template <int N, int NS, bool INV, int L>
__device__ __forceinline__ void colsplit_middle_from(float2* buf, const float2* __restrict__ tw, int t) {
  if constexpr (NS < ColSplit<N, L>::NS_LAST) {
    constexpr int E = N / L;
    constexpr int REM = N / NS;
    constexpr int RS = REM < E ? REM : E;
    float2 unused[E];
    warp_stage<N, RS, NS, INV, false, false, L>(unused, buf, tw, t);
    colsplit_middle_from<N, NS * RS, INV, L>(buf, tw, t);
  }
}
template <int N, bool INV, int L = 32>
__device__ __forceinline__ void colsplit_middle(float2* buf, const float2* __restrict__ tw, int t) {
  colsplit_middle_from<N, N / L, INV, L>(buf, tw, t);
}

// last stage of column cc: butterflies j = r0 + L q read positions j + NS r (padded index:
// (r0 + r0>>S) + (L q + (L q)>>S) + (NS + NS>>S) r), twiddle entries (r-1)*NS + j of the
// stage, and leave row j + NS r in v[q + (NS/L) r]
template <int N, bool INV, int L = 32>
__device__ __forceinline__ void colsplit_last(float2 (&v)[N / L], const float2* colbuf,
                                              const float2* __restrict__ tw, int r0) {
  constexpr int NS = ColSplit<N, L>::NS_LAST;
  constexpr int RS = N / NS;
  constexpr int Q = NS / L;
  constexpr int TWOFF = wtw_offset(N, NS, L);
  constexpr int S = pad_shift(N, L);
  float2 a[N / L];
  const float2* b = colbuf + r0 + (r0 >> S);
#pragma unroll
  for (int q = 0; q < Q; q++)
#pragma unroll
    for (int r = 0; r < RS; r++) a[q * RS + r] = b[L * q + ((L * q) >> S) + (NS + (NS >> S)) * r];
  const float2* twl = tw + TWOFF + r0;
#pragma unroll
  for (int q = 0; q < Q; q++)
#pragma unroll
    for (int r = 1; r < RS; r++) {
      float2 w = twl[(r - 1) * NS + L * q];
      if (INV) w.y = -w.y;
      a[q * RS + r] = cmul(a[q * RS + r], w);
    }
#pragma unroll
  for (int q = 0; q < Q; q++) Dft<RS, INV>::run(&a[q * RS]);
#pragma unroll
  for (int q = 0; q < Q; q++)
#pragma unroll
    for (int r = 0; r < RS; r++) v[q + r * Q] = a[q * RS + r];
}

}  // namespace bpmgb
