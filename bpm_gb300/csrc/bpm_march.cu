// Split-step beam propagation z-march on GB300 (sm_103a).
//
// Reference algorithm (per z-step i, bpm/bpm/bpm_3d.py:283-381):
//   u_hat = FFT2(u)                      (forward, unnormalised)
//   [weighted] dn0 = sum|u_hat|*dn_slice0 / sum|u_hat|          (bpm_3d.py:302-303)
//   u_hat *= h(n)                        (mult_propagator*, bpm_3d_kernels.cl:408-493)
//   u = IFFT2(u_hat)                     (normalised by 1/(nx*ny))
//   u *= exp(-i k0 dz (dn[i+1]-dn0)) * taper    (mult_dn*, bpm_3d_kernels.cl:20-283)
//   store u or |u|^2 as plane i+1        (copy_intens, bpm_3d_kernels.cl:396-404)
//
// GB300 design. FFT2 = row FFTs (along x) then column FFTs (along y). A z-step is two
// passes over the field held in a workspace W (one plane per field of the group):
//   column pass : load 16 full columns, forward column FFT, multiply by the propagator
//                 (with the 1/(nx*ny) normalisation folded in), inverse column FFT, store.
//   row pass    : load 16 full rows, inverse row FFT, phase mask of dn slice z with taper,
//                 write plane z of the output (field or |u|^2), forward row FFT of the next
//                 step, store.
// so the forward row FFT of step i+1 is fused with the inverse row FFT and mask of step i
// and nothing but the field itself makes a round trip between passes. The weighted mean
// mode needs the plane-wide sums between the forward column FFT and the propagator, so
// its column pass is split in two (forward FFT + partial sums | propagator + inverse FFT).
// Many fields (illumination angles, wavelengths) march together: grid.y indexes the
// field within a group, and a group's planes stay L2-resident between passes while the
// dn slice is read from HBM once for the whole group.
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include <cooperative_groups.h>

#include "common.cuh"
#include "fft_tile.cuh"
#include "warp_fft.cuh"

using namespace bpmgb;

static const float PI_F = 3.14159265358979f;  // bpm_3d_kernels.cl:3

// field groups a batch may march at the same time (one workspace slot and stream each):
// conc_limit() of them, 4 unless BPM_GB300_CONC (1..8) says otherwise
constexpr int kMaxConcurrentGroups = 8;
static int conc_limit() {
  static const int v = [] {
    const char* e = getenv("BPM_GB300_CONC");
    const int c = e ? atoi(e) : 4;
    return c < 1 ? 1 : (c > kMaxConcurrentGroups ? kMaxConcurrentGroups : c);
  }();
  return v;
}

struct bpm_plan {
  bpm_grid_desc d;
  int device;
  float2* tw_x;     // W_nx^k
  float2* tw_y;     // W_ny^k
  float2* wtw_x;    // stage-ordered twiddles of the warp FFT along x (64 <= nx <= 1024)
  float2* wtw_y;    // ... along y
  float* kx2;       // (2.f*M_PI*FFTFREQ(i,nx,dx))^2, FP32 recipe
  float* ky2;
  float2* H;        // unnormalised propagator table (IGNORE mean mode), (ny, nx)
  float2* Ht;       // the same table transposed, (nx, ny): a column's entries are contiguous
  float* taper;     // taper value per distance < absorbing_width
  float* sw;        // scattering weights cos(theta), (ny, nx)
  float* gw;        // g-factor weights cos(theta)^2
  float k0f, dzf, n0f, unit_k;
  double k0;
  // streams on which groups of fields march concurrently, with their fork/join events
  cudaStream_t aux[kMaxConcurrentGroups];
  cudaEvent_t ev_fork, ev_join[kMaxConcurrentGroups];
  // device->host streaming of the output volume (bpm_propagate_to_host): the copy stream,
  // one "planes ready" event per march stream, and the final join
  cudaStream_t copy;
  cudaEvent_t ev_ready[kMaxConcurrentGroups], ev_copied;
  int max_pitch;
  // false for a plan made by bpm_plan_derive: the device tables belong to its base plan
  bool owns_tables;
};

struct bpm_exec {
  cudaGraphExec_t exec;
  cudaGraph_t graph;
  unsigned long long launches;
};

namespace {

// ---------------------------------------------------------------------------------------
// host-side FP32 recipes (compiled with -ffp-contract=off: every operation rounds as written)
// ---------------------------------------------------------------------------------------
float fftfreq_f32(int i, int N, float d) {  // FFTFREQ, bpm_3d_kernels.cl:6
  int half = (N - 1) / 2 + 1;
  int num = (i < half) ? i : (i - half) - N / 2;
  float f = 1.f * (float)num;
  f = f / (float)N;
  f = f / d;
  return f;
}

// stage-ordered twiddle table of the warp FFT with L lanes per sequence (layout documented
// at wtw_offset), FP64
std::vector<float2> warp_twiddles(int N, int L = 32) {
  std::vector<float2> w(wtw_size(N, L));
  const int E = N / L;
  int ns = 1;
  while (ns < N) {
    const int rs = std::min(E, N / ns);
    if (ns > 1) {
      const int off = wtw_offset(N, ns, L);
      for (int r = 1; r < rs; r++)
        for (int jm = 0; jm < ns; jm++) {
          const double a = -2. * M_PI * (double)((long)jm * r * (N / (ns * rs))) / N;
          w[off + (r - 1) * ns + jm] = make_float2((float)cos(a), (float)sin(a));
        }
    }
    ns *= rs;
  }
  return w;
}

float taper_value(int dist, int absorb) {  // bpm_3d_kernels.cl:36
  float arg = PI_F * (float)dist;
  arg = arg / (float)absorb;
  float c = cosf(arg);
  return 0.5f * (1.f - c);
}

// ---------------------------------------------------------------------------------------
// plan tables on the device (FP64 arithmetic)
// ---------------------------------------------------------------------------------------
__global__ void build_tables_kernel(int nx, int ny, double dx, double dy, double dz, double n0,
                                    double k0, float n0f, float k0f, int prop_kind, int fresnel,
                                    const float* __restrict__ kx2, const float* __restrict__ ky2,
                                    float2* __restrict__ H, float2* __restrict__ Ht, float* __restrict__ sw,
                                    float* __restrict__ gw) {
  int x = blockIdx.x * blockDim.x + threadIdx.x;
  int y = blockIdx.y;
  if (x >= nx) return;
  // FP64 k-grid, 2*pi*fftfreq (numpy)
  const double twopi = 6.283185307179586476925286766559;
  double fx = (x < (nx + 1) / 2) ? (double)x : (double)(x - nx);
  double fy = (y < (ny + 1) / 2) ? (double)y : (double)(y - ny);
  double kx = twopi * fx / (nx * dx);
  double ky = twopi * fy / (ny * dy);
  double tmp64 = n0 * n0 * k0 * k0 - kx * kx - ky * ky;
  bool prop;
  if (prop_kind == BPM_PROP_FUNCTIONAL) {
    // evanescent mask of compute_propagator: FP32 recipe, no contraction
    float nk = __fmul_rn(__fmul_rn(__fmul_rn(n0f, n0f), k0f), k0f);
    float tmp = __fsub_rn(__fsub_rn(nk, kx2[x]), ky2[y]);
    prop = tmp >= 0.f;
  } else {
    prop = tmp64 >= 0.0;  // host FP64 propagator: NaN where negative
  }
  double kz = tmp64 > 0.0 ? sqrt(tmp64) : 0.0;
  double ph = -dz * kz;
  double s, c;
  sincos(ph, &s, &c);
  const float2 hv = prop ? make_float2((float)c, (float)s) : make_float2(0.f, 0.f);
  H[(size_t)y * nx + x] = hv;
  Ht[(size_t)x * ny + y] = hv;
  // scattering weights (bpm_3d.py:227-244): cos(theta) = real(H0)/n0/k0 with the FP64 host H0
  double h0 = tmp64 >= 0.0 ? sqrt(tmp64) : 0.0;
  if (fresnel) h0 = n0 * k0 - .5 * (kx * kx + ky * ky) / n0 / k0;
  double ct = h0 / n0 / k0;
  sw[(size_t)y * nx + x] = (float)ct;
  gw[(size_t)y * nx + x] = (float)(ct * ct);
}

// ---------------------------------------------------------------------------------------
// kernels
// ---------------------------------------------------------------------------------------
struct RowParams {
  const float2* src;        // group's input planes (u0 + b0*plane, or W)
  long long src_bstride;    // float2 elements between fields
  float2* W;                // group workspace planes
  int nx, ny, nz, z;        // z = plane produced by this pass (dn slice index)
  int do_inv, do_fwd, do_mask;
  const void* dn;           // dn of field 0 of the group
  int dn_dtype;
  long long dn_bstride;     // elements
  float unit_k;
  int absorb;
  const float* taper;
  int mean_mode;
  const float* dn0_field;   // weighted: per group field
  const float* slice_dn0;   // simple: per slice
  void* out;                // output of field 0 of the group
  int out_kind;
  long long out_bstride;    // elements
  int zout0;                // output plane index = z - zout0
  float2* last_plane;       // group's exit planes or NULL
  float2* ckpt;             // group's checkpoint planes (G, n_ckpt, ny, nx) or NULL
  int ckpt_every, n_ckpt;
  const float* scat_part;   // [G][ntiles][2]
  int n_ctiles;
  float* scat_p;            // group's (nz) rows
  float* scat_g;
  float prefac_f;
  const float2* tw;
  const float2* wtw;        // stage-ordered twiddles of the warp FFT
  // adjoint passes only
  const float2* seg;        // forward fields of the current segment (G, planes, ny, nx)
  long long seg_bstride;    // float2 elements between fields
  int seg_z0;               // plane index of the segment's first plane
  float* grad_dn;           // group's (nz, ny, nx) dn gradients
  float2* grad_u0;          // group's (ny, nx) u0 gradients or NULL
  const float2* mask;       // precomputed masks of the shared dn, (nz, ny, nx), or NULL
  // adjoint with the dn gradient summed over the fields (row_adj_shared_kernel, grad_sum 1):
  // block 0 of a row writes its fields' sum to grad_dn, block b >= 1 to grad_part + (b - 1) *
  // grad_part_stride, stored (grad_acc 0, the first group of the request) or added (grad_acc
  // 1, the later groups)
  int grad_sum;
  float* grad_part;
  long long grad_part_stride;
  int grad_acc;
};

__device__ __forceinline__ float load_dn_real(const void* dn, int dtype, size_t idx) {
  if (dtype == BPM_DN_F16) return __half2float(reinterpret_cast<const __half*>(dn)[idx]);
  return __ldg(reinterpret_cast<const float*>(dn) + idx);
}

// The pointwise work of a row pass on one element v = u(x, y) of plane z, shared by the
// tile and warp row kernels. Forward: phase mask of dn slice z (+ taper) and the plane-z
// outputs. Adjoint: dn gradient against the forward field, conjugate mask; at plane 0 the
// adjoint value is the u0 gradient.
// Phase mask of dn slice z at (x, y): M = taper * exp(-i k0 dz dn) for real dn
// (mult_dn*, bpm_3d_kernels.cl:20-81, 198-262), exp(k0 dz Im dn) * exp(-i k0 dz Re dn) with
// no taper for complex dn (mult_dn*_complex, :84-101, :265-283). The mean-index shift dn0
// enters as the separate factor exp(+i k0 dz dn0) (row_rot), so M depends on dn alone and
// can be computed once per dn volume for a whole batch (bpm_mask_precompute); the on-the-fly
// and precomputed masks are the same FP32 arithmetic, bit for bit.
__device__ __forceinline__ float2 mask_from_complex(float2 d, float unit_k) {
  float s, c;
  const float m = expf(unit_k * d.y);
  sincosf((-unit_k) * d.x, &s, &c);
  return make_float2(m * c, m * s);
}

__device__ __forceinline__ float2 mask_from_real(float dnv, float unit_k, int x, int y, int nx, int ny, int absorb,
                                                 const float* taper) {
  float s, c;
  sincosf((-unit_k) * dnv, &s, &c);
  float2 M = make_float2(c, s);
  const int dist = min(min(nx - 1 - x, x), min(ny - 1 - y, y));
  if (dist < absorb) {
    const float a = taper[dist];
    M.x *= a;
    M.y *= a;
  }
  return M;
}

__device__ __forceinline__ float2 mask_value(const void* dn, int dtype, size_t idx, float unit_k, int x, int y,
                                             int nx, int ny, int absorb, const float* taper) {
  if (dtype == BPM_DN_C64) return mask_from_complex(__ldg(reinterpret_cast<const float2*>(dn) + idx), unit_k);
  return mask_from_real(load_dn_real(dn, dtype, idx), unit_k, x, y, nx, ny, absorb, taper);
}

// PRE = 1: the masks come precomputed (p.mask); PRE = 0: formed on the fly from dn. The
// two are compiled separately so the precomputed kernel carries no sincosf.
template <int PRE>
__device__ __forceinline__ float2 row_mask(const RowParams& p, int x, int y, int gl, size_t zoff, size_t pix) {
  if constexpr (PRE == 1) {
    return p.mask[zoff + pix];
  } else {
    return mask_value(p.dn, p.dn_dtype, gl * p.dn_bstride + zoff + pix, p.unit_k, x, y, p.nx, p.ny, p.absorb,
                      p.taper);
  }
}

// exp(+i k0 dz dn0), the mean-index shift of the mask (identity when dn0 = 0)
__device__ __forceinline__ float2 row_rot(const RowParams& p, float dn0) {
  float s, c;
  sincosf(p.unit_k * dn0, &s, &c);
  return make_float2(c, s);
}

template <bool ADJ, int PRE>
__device__ __forceinline__ float2 row_point(const RowParams& p, float2 v, int x, int y, int gl, size_t plane,
                                            size_t zoff, size_t ooff, float dn0, float2 rot, bool last,
                                            float2* ckp) {
  const size_t pix = (size_t)y * p.nx + x;
  if (ADJ) {
    if (p.z == 0) {
      if (p.grad_u0) p.grad_u0[gl * plane + pix] = v;
      return v;
    }
    if (p.do_mask) {
      const float2 u = p.seg[gl * p.seg_bstride + (size_t)(p.z - p.seg_z0) * plane + pix];
      p.grad_dn[(size_t)gl * p.nz * plane + zoff + pix] = p.unit_k * fmaf(v.x, u.y, -(v.y * u.x));
      const float2 M = row_mask<PRE>(p, x, y, gl, zoff, pix);
      v = cmul(v, make_float2(M.x, -M.y));
      if (dn0 != 0.f) v = cmul(v, make_float2(rot.x, -rot.y));
    }
    return v;
  }
  if (p.do_mask) {
    v = cmul(v, row_mask<PRE>(p, x, y, gl, zoff, pix));
    if (dn0 != 0.f) v = cmul(v, rot);
  }
  if (p.out_kind == BPM_OUT_FIELD)
    __stcs(reinterpret_cast<float2*>(p.out) + gl * p.out_bstride + ooff + pix, v);
  else if (p.out_kind == BPM_OUT_INTENSITY)
    __stcs(reinterpret_cast<float*>(p.out) + gl * p.out_bstride + ooff + pix, cabs2(v));
  if (last && p.last_plane) p.last_plane[gl * plane + pix] = v;
  if (ckp) ckp[pix] = v;
  return v;
}

// precomputed phase masks of a shared dn volume, (nz, ny, nx) complex64
__global__ void mask_precompute_kernel(const void* dn, int dtype, float unit_k, int nx, int ny, int absorb,
                                       const float* taper, float2* mask) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y, z = blockIdx.z;
  if (x >= nx) return;
  const size_t idx = ((size_t)z * ny + y) * nx + x;
  __stcs(mask + idx, mask_value(dn, dtype, idx, unit_k, x, y, nx, ny, absorb, taper));
}

// dn0 of the current field and plane: the weighted-mode per-field value or the simple-mode
// slice mean (0 in "ignore")
__device__ __forceinline__ float row_dn0(const RowParams& p, int gl) {
  if (p.mean_mode == BPM_MEAN_WEIGHTED && p.dn0_field) return p.dn0_field[gl];
  if (p.mean_mode == BPM_MEAN_SIMPLE && p.slice_dn0) return p.slice_dn0[p.z];
  return 0.f;
}

// the scattering sums of step z, finished by one thread of the first block of each field
__device__ __forceinline__ void row_scatter_finish(const RowParams& p, int gl) {
  float* prow = p.scat_p + (size_t)gl * p.nz;
  float* grow = p.scat_g ? p.scat_g + (size_t)gl * p.nz : nullptr;
  if (p.z == 0) {
    prow[0] = 0.f;
    if (grow) grow[0] = __fdiv_rn(0.f, 0.f);
    return;
  }
  const float* part = p.scat_part + (size_t)gl * p.n_ctiles * 2;
  float S = 0.f, G = 0.f;
  for (int t = 0; t < p.n_ctiles; t++) {
    S += part[2 * t];
    G += part[2 * t + 1];
  }
  const float pv = p.prefac_f * S;
  prow[p.z] = pv;
  if (grow) grow[p.z] = __fdiv_rn(p.prefac_f * G, pv);
}

// Row pass over 16 rows of one field. Forward (ADJ = false): [inverse row FFT], phase mask
// of slice z with taper, plane-z outputs, [forward row FFT]. Adjoint (ADJ = true): [inverse
// row FFT] of the adjoint field, dn gradient k0 dz Im(conj(G) u_z) against the forward field
// u_z of the segment, conjugate mask, [forward row FFT]; at plane 0 the adjoint is the u0
// gradient.
template <int N, bool ADJ>
__global__ void __launch_bounds__(TileCfg<N>::THREADS, TileCfg<N>::MINB)
row_pass_kernel(RowParams p) {
  constexpr int T = TileCfg<N>::THREADS;
  constexpr int R = TileCfg<N>::R;
  extern __shared__ float2 smem[];
  float2* tile = smem;
  float2* tw = smem + N * 16;
  const int tid = threadIdx.x;
  const int gl = blockIdx.y;
  const int y0 = blockIdx.x * 16;
  const size_t plane = (size_t)N * p.ny;

  // the 16 rows are contiguous in memory: element e = r*N + x; each thread holds R of them
  constexpr int PER = 16 * N / T;
  if (p.do_inv || p.do_fwd)
    for (int k = tid; k < N; k += T) tw[k] = p.tw[k];
  dep_wait();
  dep_release();
  {
    const float2* src = p.src + gl * p.src_bstride + (size_t)y0 * N;
    float2 buf[PER];
#pragma unroll
    for (int i = 0; i < PER; i++) buf[i] = src[tid + i * T];
#pragma unroll
    for (int i = 0; i < PER; i++) {
      const int e = tid + i * T;
      tile[tile_idx(e % N, e / N)] = buf[i];
    }
  }
  __syncthreads();

  if (p.do_inv) tile_fft<N, R, true>(tile, tw);

  // pointwise work, one element per thread and iteration, consecutive x across a warp
  const float dn0 = row_dn0(p, gl);
  const float2 rot = row_rot(p, dn0);
  const bool last = (p.z == p.nz - 1);
  const size_t zoff = (size_t)p.z * plane;
  const size_t ooff = (size_t)(p.z - p.zout0) * plane;
  float2* ckp = nullptr;
  if (!ADJ && p.ckpt && p.z % p.ckpt_every == 0)
    ckp = p.ckpt + ((size_t)gl * p.n_ckpt + p.z / p.ckpt_every) * plane;
#pragma unroll 4
  for (int i = 0; i < PER; i++) {
    const int e = tid + i * T;
    const int r = e / N;
    const int x = e % N;
    const float2 v = p.mask
        ? row_point<ADJ, 1>(p, tile[tile_idx(x, r)], x, y0 + r, gl, plane, zoff, ooff, dn0, rot, last, ckp)
        : row_point<ADJ, 0>(p, tile[tile_idx(x, r)], x, y0 + r, gl, plane, zoff, ooff, dn0, rot, last, ckp);
    if (p.do_mask) tile[tile_idx(x, r)] = v;
  }
  if (!ADJ && p.scat_p && blockIdx.x == 0 && tid == 0) row_scatter_finish(p, gl);

  if (!p.do_fwd) return;
  __syncthreads();
  tile_fft<N, R, false>(tile, tw);
  float2* dst = p.W + gl * plane + (size_t)y0 * N;
#pragma unroll
  for (int i = 0; i < PER; i++) {
    const int e = tid + i * T;
    dst[e] = tile[tile_idx(e % N, e / N)];
  }
}

struct ColParams {
  float2* W;
  int nx, ny, nz, z;         // z = step index: the field goes from plane z to z+1
  int prop_mode;             // 0 = table H, 1 = FP32 recipe with slice_n[z+1], 2 = weighted
  const float2* H;
  const float2* Ht;          // H transposed (nx, ny), for the warp column kernels
  const float* kx2;
  const float* ky2;
  float k0f, dzf, n00f;
  const float* slice_n;
  float scale;               // 1/(nx*ny)
  const void* dn;            // weighted: dn of field 0 of the group (slice 0 is used)
  int dn_dtype;
  long long dn_bstride;
  float* red_part;           // [G][ntiles][2]
  float* dn0_field;          // [G]
  int scat;
  const float* sw;
  const float* gw;
  float* scat_part;          // [G][ntiles][2]
  double plain_phase;        // k0*n0*dz
  int spi;                   // scattering_plane_ind
  int conj_h;                // adjoint: multiply by conj(H)
  const float2* tw;
  const float2* wtw;         // stage-ordered twiddles of the warp FFT
  int dn_stage;              // weighted: dn rows may be staged with 16-byte cp.async
  int col_block;             // 0: the library's rule; 4, 8 or 16 columns per non-weighted block
  int col_fuse;              // weighted: 1 one fused column pass where available, 0 or 2 two passes
};

template <int T>
__device__ __forceinline__ void block_sum2(float& a, float& b, float* red) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    a += __shfl_xor_sync(0xffffffffu, a, o);
    b += __shfl_xor_sync(0xffffffffu, b, o);
  }
  constexpr int NW = (T + 31) / 32;
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) {
    red[2 * w] = a;
    red[2 * w + 1] = b;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    float s = 0.f, t = 0.f;
    for (int i = 0; i < NW; i++) {
      s += red[2 * i];
      t += red[2 * i + 1];
    }
    a = s;
    b = t;
  }
}

template <int N, int T = TileCfg<N>::THREADS>
__device__ __forceinline__ void col_load(float2* tile, const float2* Wp, int nx, int x0) {
  constexpr int PER = 16 * N / T;
  float2 buf[PER];
#pragma unroll
  for (int i = 0; i < PER; i++) {
    const int e = threadIdx.x + i * T;
    buf[i] = Wp[(size_t)(e >> 4) * nx + x0 + (e & 15)];
  }
#pragma unroll
  for (int i = 0; i < PER; i++) {
    const int e = threadIdx.x + i * T;
    tile[tile_idx(e >> 4, e & 15)] = buf[i];
  }
}

template <int N, int T = TileCfg<N>::THREADS>
__device__ __forceinline__ void col_store(const float2* tile, float2* Wp, int nx, int x0) {
  constexpr int PER = 16 * N / T;
#pragma unroll
  for (int i = 0; i < PER; i++) {
    const int e = threadIdx.x + i * T;
    Wp[(size_t)(e >> 4) * nx + x0 + (e & 15)] = tile[tile_idx(e >> 4, e & 15)];
  }
}

// plain_wave_dct[z+1] = nx*ny*exp(-i k0 n0 (spi + z+1) dz) of bpm_3d.py:253, FP64 then complex64
__device__ __forceinline__ float2 plain_wave(const ColParams& p) {
  double ph = -p.plain_phase * (double)(p.spi + p.z + 1);
  double s, c;
  sincos(ph, &s, &c);
  double m = (double)p.nx * (double)p.ny;
  return make_float2((float)(m * c), (float)(m * s));
}

// k-space element (kx index x, ky index y) times the propagator, with the scattering partial
// sums of bpm_3d.py:335-341 and the 1/(nx*ny) inverse-FFT normalisation folded in
// COLUMN: the caller walks one column (x fixed, y over the lanes) and reads the transposed
// table; ky2: the ky^2 table, in global or shared memory
// htcol (COLUMN only, optional): the column's entries of the transposed table, staged
template <bool COLUMN = false>
__device__ __forceinline__ float2 prop_point(const ColParams& p, float2 v, int x, int y, float nk, float2 plain,
                                             float& S, float& G, const float* ky2,
                                             const float2* htcol = nullptr) {
  float2 h;
  if (p.prop_mode == 0) {
    h = COLUMN ? (htcol ? htcol[y] : __ldg(p.Ht + (size_t)x * p.ny + y)) : __ldg(p.H + (size_t)y * p.nx + x);
    if (p.conj_h) h.y = -h.y;
  } else {
    const float tmp = __fsub_rn(__fsub_rn(nk, __ldg(p.kx2 + x)), ky2[y]);
    if (tmp >= 0.f) {
      const float ph = __fmul_rn(-p.dzf, __fsqrt_rn(tmp));
      sincosf(ph, &h.y, &h.x);
    } else {
      h = make_float2(0.f, 0.f);
    }
  }
  v = cmul(v, h);
  if (p.scat) {
    float2 d = v;
    if (x == 0 && y == 0) d = csub(d, plain);
    const float a2 = cabs2(d);
    const size_t k = (size_t)y * p.nx + x;
    S = fmaf(__ldg(p.sw + k), a2, S);
    G = fmaf(__ldg(p.gw + k), a2, G);
  }
  return cscale(v, p.scale);
}

// n*n*k0*k0 in the FP32 order of the kernels (bpm_3d_kernels.cl:425), no contraction
__device__ __forceinline__ float prop_nk(const ColParams& p, float n_eff) {
  return __fmul_rn(__fmul_rn(__fmul_rn(n_eff, n_eff), p.k0f), p.k0f);
}

template <int T>
__device__ __forceinline__ void scat_partials_store(const ColParams& p, float S, float G, int gl, float* red) {
  block_sum2<T>(S, G, red);
  if (threadIdx.x == 0) {
    float* o = p.scat_part + ((size_t)gl * (p.nx / 16) + blockIdx.x) * 2;
    o[0] = S;
    o[1] = G;
  }
}

// multiply the k-space column tile by the propagator (+ scattering partial sums)
template <int N>
__device__ __forceinline__ void col_propagate(float2* tile, const ColParams& p, float n_eff, int x0,
                                              int gl, float* red) {
  constexpr int T = TileCfg<N>::THREADS;
  const float nk = prop_nk(p, n_eff);
  float S = 0.f, G = 0.f;
  const float2 plain = (p.scat && x0 == 0) ? plain_wave(p) : make_float2(0.f, 0.f);
  for (int e = threadIdx.x; e < 16 * N; e += T) {
    const int y = e >> 4;
    const int c = e & 15;
    tile[tile_idx(y, c)] = prop_point(p, tile[tile_idx(y, c)], x0 + c, y, nk, plain, S, G, p.ky2);
  }
  if (p.scat) scat_partials_store<T>(p, S, G, gl, red);
  __syncthreads();
}

// non-weighted column pass: forward FFT, propagator, inverse FFT
template <int N>
__global__ void __launch_bounds__(TileCfg<N>::THREADS, TileCfg<N>::MINB)
col_pass_kernel(ColParams p) {
  constexpr int R = TileCfg<N>::R;
  extern __shared__ float2 smem[];
  float2* tile = smem;
  float2* tw = smem + N * 16;
  __shared__ float red[64];
  const int gl = blockIdx.y;
  const int x0 = blockIdx.x * 16;
  float2* Wp = p.W + (size_t)gl * p.nx * N;
  for (int k = threadIdx.x; k < N; k += TileCfg<N>::THREADS) tw[k] = p.tw[k];
  dep_wait();
  dep_release();
  col_load<N>(tile, Wp, p.nx, x0);
  __syncthreads();
  tile_fft<N, R, false>(tile, tw);
  float n_eff = p.n00f;
  if (p.prop_mode == 1) n_eff = p.slice_n[p.z + 1];
  col_propagate<N>(tile, p, n_eff, x0, gl, red);
  tile_fft<N, R, true>(tile, tw);
  col_store<N>(tile, Wp, p.nx, x0);
}

// weighted mode, part 1: forward column FFT and the partial sums of |u_hat|*dn0, |u_hat|
template <int N>
__global__ void __launch_bounds__(TileCfg<N>::THREADS, TileCfg<N>::MINB)
col_fwd_reduce_kernel(ColParams p) {
  constexpr int T = TileCfg<N>::THREADS;
  constexpr int R = TileCfg<N>::R;
  extern __shared__ float2 smem[];
  float2* tile = smem;
  float2* tw = smem + N * 16;
  __shared__ float red[64];
  const int gl = blockIdx.y;
  const int x0 = blockIdx.x * 16;
  float2* Wp = p.W + (size_t)gl * p.nx * N;
  for (int k = threadIdx.x; k < N; k += T) tw[k] = p.tw[k];
  dep_wait();
  dep_release();
  col_load<N>(tile, Wp, p.nx, x0);
  __syncthreads();
  tile_fft<N, R, false>(tile, tw);
  float sdn = 0.f, su = 0.f;
  for (int e = threadIdx.x; e < 16 * N; e += T) {
    const int y = e >> 4;
    const int c = e & 15;
    const float2 v = tile[tile_idx(y, c)];
    const float a = __fsqrt_rn(cabs2(v));
    su += a;
    if (p.dn) sdn = fmaf(a, load_dn_real(p.dn, p.dn_dtype, gl * p.dn_bstride + (size_t)y * p.nx + x0 + c), sdn);
  }
  block_sum2<T>(sdn, su, red);
  if (threadIdx.x == 0) {
    float* o = p.red_part + ((size_t)gl * (p.nx / 16) + blockIdx.x) * 2;
    o[0] = sdn;
    o[1] = su;
  }
  col_store<N>(tile, Wp, p.nx, x0);
}

// weighted mode, part 2: n = n00 + dn_sum/u_sum, propagator, inverse column FFT
template <int N>
__global__ void __launch_bounds__(TileCfg<N>::THREADS, TileCfg<N>::MINB)
col_inv_kernel(ColParams p) {
  constexpr int R = TileCfg<N>::R;
  extern __shared__ float2 smem[];
  float2* tile = smem;
  float2* tw = smem + N * 16;
  __shared__ float red[64];
  __shared__ float s_n;
  const int gl = blockIdx.y;
  const int x0 = blockIdx.x * 16;
  float2* Wp = p.W + (size_t)gl * p.nx * N;
  for (int k = threadIdx.x; k < N; k += TileCfg<N>::THREADS) tw[k] = p.tw[k];
  dep_wait();
  dep_release();
  if (threadIdx.x == 0) {
    // every block of the field sums the partials in the same order: identical results
    const float* part = p.red_part + (size_t)gl * (p.nx / 16) * 2;
    float dn_sum = 0.f, u_sum = 0.f;
    for (int t = 0; t < p.nx / 16; t++) {
      dn_sum += part[2 * t];
      u_sum += part[2 * t + 1];
    }
    const float dn0 = dn_sum / u_sum;  // mult_dn_mean_buff, bpm_3d_kernels.cl:117
    s_n = p.n00f + dn0;                // mult_propagator_buff, bpm_3d_kernels.cl:482
    if (blockIdx.x == 0) p.dn0_field[gl] = dn0;
  }
  col_load<N>(tile, Wp, p.nx, x0);
  __syncthreads();
  col_propagate<N>(tile, p, s_n, x0, gl, red);
  tile_fft<N, R, true>(tile, tw);
  col_store<N>(tile, Wp, p.nx, x0);
}

// ---------------------------------------------------------------------------------------
// sequence-in-registers kernels (128 <= N <= 1024): L lanes (a warp, or a half-warp for
// 512-point sequences) transform one row or one column entirely in registers, exchanging
// only through the sequence's own shared-memory buffer
// ---------------------------------------------------------------------------------------
constexpr int kRowWarps = 8;   // rows per block
constexpr int kColWarps = 16;  // columns per block (16 columns = one 128-byte segment per row)

template <int N, int L = 32>
struct WarpCfg {
  static constexpr size_t row_smem(int rw) {
    return ((size_t)N + (size_t)rw * WarpFft<N, L>::BUF) * sizeof(float2);
  }
  static constexpr size_t ROW_SMEM = row_smem(kRowWarps);
  static constexpr size_t ROW_SMEM_SHARED = ROW_SMEM + (size_t)N * sizeof(float2);  // + the staged row
  // row_adj_shared_kernel with `slots` sequences: + a forward-field row and a row of
  // gradient terms per sequence
  static constexpr size_t adj_smem(int slots) {
    return row_smem(slots) + (size_t)N * sizeof(float2) + (size_t)slots * N * (sizeof(float2) + sizeof(float));
  }
};

// blocks per SM a row kernel of RW sequences of L lanes must fit: 32 values per lane need
// up to 128 registers a thread, fewer 64 (85 for the on-the-fly mask)
__host__ __device__ constexpr int row_min_blocks(int N, int L, int PRE, int RW) {
  return N / L >= 32 ? 65536 / (128 * RW * L) : (PRE ? 4 : 3) * (kRowWarps / RW);
}

// Row pass, L lanes per row: coalesced row load straight into registers, [inverse row
// FFT], pointwise work, [forward row FFT], coalesced store. No block-level barrier after
// the twiddle table is loaded.
template <int N, bool ADJ, int PRE, int RW = kRowWarps, int L = 32>
__global__ void __launch_bounds__(RW * L, row_min_blocks(N, L, PRE, RW))
row_warp_kernel(RowParams p) {
  constexpr int E = N / L;
  constexpr int T = RW * L;
  extern __shared__ float2 smem[];
  float2* tw = smem;
  const int seq = threadIdx.x / L, t = threadIdx.x % L;
  float2* buf = smem + N + seq * WarpFft<N, L>::BUF;
  const int gl = blockIdx.y;
  const int y = blockIdx.x * RW + seq;
  const size_t plane = (size_t)N * p.ny;
  // the twiddle table (a plan constant) is fetched before the wait for the previous pass;
  // the row loads go out before the barrier, so their latency overlaps the table's
  const bool fft = p.do_inv || p.do_fwd;
  if (fft)
    for (int k = threadIdx.x; k < WarpFft<N, L>::TW; k += T) tw[k] = p.wtw[k];
  dep_wait();
  dep_release();
  float2 v[E];
  const float2* src = p.src + gl * p.src_bstride + (size_t)y * N;
#pragma unroll
  for (int m = 0; m < E; m++) v[m] = src[t + L * m];
  if (fft) __syncthreads();
  if (p.do_inv) warp_fft<N, true, L>(v, buf, tw, t);

  const float dn0 = row_dn0(p, gl);
  const float2 rot = row_rot(p, dn0);
  const bool last = (p.z == p.nz - 1);
  const size_t zoff = (size_t)p.z * plane;
  const size_t ooff = (size_t)(p.z - p.zout0) * plane;
  float2* ckp = nullptr;
  if (!ADJ && p.ckpt && p.z % p.ckpt_every == 0)
    ckp = p.ckpt + ((size_t)gl * p.n_ckpt + p.z / p.ckpt_every) * plane;
#pragma unroll
  for (int m = 0; m < E; m++)
    v[m] = row_point<ADJ, PRE>(p, v[m], t + L * m, y, gl, plane, zoff, ooff, dn0, rot, last, ckp);
  if (!ADJ && p.scat_p && blockIdx.x == 0 && threadIdx.x == 0) row_scatter_finish(p, gl);

  if (!p.do_fwd) return;
  warp_fft<N, false, L>(v, buf, tw, t);
  float2* dst = p.W + gl * plane + (size_t)y * N;
#pragma unroll
  for (int m = 0; m < E; m++) dst[t + L * m] = v[m];
}

// the phase mask at (x, y) from the staged row: the precomputed mask or the dn value
template <int PRE>
__device__ __forceinline__ float2 staged_mask(const RowParams& p, const void* mland, int x, int y) {
  if constexpr (PRE == 1) {
    return static_cast<const float2*>(mland)[x];
  } else {
    if (p.dn_dtype == BPM_DN_C64) return mask_from_complex(static_cast<const float2*>(mland)[x], p.unit_k);
    const float d = p.dn_dtype == BPM_DN_F16 ? __half2float(static_cast<const __half*>(mland)[x])
                                             : static_cast<const float*>(mland)[x];
    return mask_from_real(d, p.unit_k, x, y, p.nx, p.ny, p.absorb, p.taper);
  }
}

// Forward row pass when the fields of the group share one mask (precomputed, or one dn
// volume): block (y, b) takes row y of fields fw*b .. fw*b + fw-1, L lanes per field (fw <= 8,
// chosen so no block holds idle sequences' registers; with half-warps an odd fw leaves one
// idle slot), so the mask row (or dn row) of slice z is staged once per block into shared
// memory with cp.async at block start and is ready when the sequences finish their inverse
// row FFTs. The arithmetic is row_warp_kernel's.
template <int N, int PRE, int L = 32, int FW = 0>
__global__ void __launch_bounds__(kRowWarps * 32, N / L >= 32 ? 2 : 4)
row_shared_kernel(RowParams p, int nfields, int fw_rt) {
  constexpr int E = N / L;
  // FW > 0: a compile-time block of FW fields (the full groups of batched marches), so the
  // staging loops and slot offsets are constants; FW = 0: fw_rt fields per block
  const int fw = FW > 0 ? FW : fw_rt;
  const int T = FW > 0 ? (FW * L + 31) / 32 * 32 : (int)blockDim.x;
  const int slots = T / L;
  extern __shared__ __align__(16) float2 smem[];
  float2* tw = smem;
  const int seq = threadIdx.x / L, t = threadIdx.x % L;
  float2* buf = smem + N + seq * WarpFft<N, L>::BUF;
  float2* mrow = smem + N + slots * WarpFft<N, L>::BUF;  // N float2: the staged mask or dn row
  const int y = blockIdx.x;
  const int gl = blockIdx.y * fw + seq;
  const bool active = seq < fw && gl < nfields;
  const size_t plane = (size_t)N * p.ny;
  const size_t zoff = (size_t)p.z * plane;
  for (int k = threadIdx.x; k < WarpFft<N, L>::TW; k += T) tw[k] = p.wtw[k];  // plan constant
  dep_wait();
  dep_release();
  {
    const int es = PRE ? 8 : (p.dn_dtype == BPM_DN_C64 ? 8 : (p.dn_dtype == BPM_DN_F16 ? 2 : 4));
    const char* srcm = PRE ? reinterpret_cast<const char*>(p.mask + zoff + (size_t)y * N)
                           : static_cast<const char*>(p.dn) + (zoff + (size_t)y * N) * es;
    char* dstm = reinterpret_cast<char*>(mrow);
    for (int o = threadIdx.x * 16; o < N * es; o += T * 16) cp_async16(dstm + o, srcm + o);
    cp_async_commit();
  }
  float2 v[E];
  if (active) {
    const float2* src = p.src + gl * p.src_bstride + (size_t)y * N;
#pragma unroll
    for (int m = 0; m < E; m++) v[m] = src[t + L * m];
  }
  __syncthreads();
  if (active && p.do_inv) warp_fft<N, true, L>(v, buf, tw, t);
  cp_async_wait<0>();
  __syncthreads();  // the staged row is visible to every warp
  if (!active) return;

  const float dn0 = row_dn0(p, gl);
  const float2 rot = row_rot(p, dn0);
  const bool last = (p.z == p.nz - 1);
  const size_t ooff = (size_t)(p.z - p.zout0) * plane;
  float2* ckp = nullptr;
  if (p.ckpt && p.z % p.ckpt_every == 0) ckp = p.ckpt + ((size_t)gl * p.n_ckpt + p.z / p.ckpt_every) * plane;
#pragma unroll
  for (int m = 0; m < E; m++) {
    const int x = t + L * m;
    const size_t pix = (size_t)y * N + x;
    float2 u = cmul(v[m], staged_mask<PRE>(p, mrow, x, y));
    if (dn0 != 0.f) u = cmul(u, rot);
    if (p.out_kind == BPM_OUT_FIELD)
      __stcs(reinterpret_cast<float2*>(p.out) + gl * p.out_bstride + ooff + pix, u);
    else if (p.out_kind == BPM_OUT_INTENSITY)
      __stcs(reinterpret_cast<float*>(p.out) + gl * p.out_bstride + ooff + pix, cabs2(u));
    if (last && p.last_plane) p.last_plane[gl * plane + pix] = u;
    if (ckp) ckp[pix] = u;
    v[m] = u;
  }
  if (p.scat_p && y == 0 && t == 0) row_scatter_finish(p, gl);
  if (!p.do_fwd) return;
  warp_fft<N, false, L>(v, buf, tw, t);
  float2* dst = p.W + gl * plane + (size_t)y * N;
#pragma unroll
  for (int m = 0; m < E; m++) dst[t + L * m] = v[m];
}

// Adjoint row pass for fields sharing one dn with the dn gradient summed over them (plane z
// >= 1, do_mask): block (y, b) takes row y of fields fw*b .. fw*b + fw-1, one warp each (fw <=
// 8). At block start cp.async stages the slice-z mask row (precomputed mask, or dn row) and
// every warp's row of the forward field at plane z (from the recomputed segment), so their
// reads overlap the inverse row FFT (the per-element reads of row_warp_kernel follow it);
// each warp leaves its gradient terms k0 dz Im(conj(G) u) in shared memory, and the block adds
// them over its fields in warp order, so the sum is the same in every run. The arithmetic per
// element is row_point's.
template <int N, int PRE, int L = 32>
__global__ void __launch_bounds__(kRowWarps * 32, 2)
row_adj_shared_kernel(RowParams p, int nfields, int fw) {
  constexpr int E = N / L;
  const int T = blockDim.x;
  const int slots = T / L;
  extern __shared__ __align__(16) float2 smem[];
  float2* tw = smem;
  const int seq = threadIdx.x / L, t = threadIdx.x % L;
  float2* buf = smem + N + seq * WarpFft<N, L>::BUF;
  float2* mrow = smem + N + slots * WarpFft<N, L>::BUF;  // N float2: the staged mask or dn row
  float2* srow = mrow + N;                                // slots x N float2: forward-field rows
  float* grow = reinterpret_cast<float*>(srow + (size_t)slots * N);  // slots x N gradient terms
  const int y = blockIdx.x;
  const int gl = blockIdx.y * fw + seq;
  const bool active = seq < fw && gl < nfields;
  const size_t plane = (size_t)N * p.ny;
  const size_t zoff = (size_t)p.z * plane;
  for (int k = threadIdx.x; k < WarpFft<N, L>::TW; k += T) tw[k] = p.wtw[k];  // plan constant
  dep_wait();
  dep_release();
  {
    const int es = PRE ? 8 : (p.dn_dtype == BPM_DN_F16 ? 2 : 4);
    const char* srcm = PRE ? reinterpret_cast<const char*>(p.mask + zoff + (size_t)y * N)
                           : static_cast<const char*>(p.dn) + (zoff + (size_t)y * N) * es;
    char* dstm = reinterpret_cast<char*>(mrow);
    for (int o = threadIdx.x * 16; o < N * es; o += T * 16) cp_async16(dstm + o, srcm + o);
    if (active) {
      const char* srcs = reinterpret_cast<const char*>(p.seg + gl * p.seg_bstride +
                                                       (size_t)(p.z - p.seg_z0) * plane + (size_t)y * N);
      char* dsts = reinterpret_cast<char*>(srow + (size_t)seq * N);
      for (int o = t * 16; o < N * 8; o += L * 16) cp_async16(dsts + o, srcs + o);
    }
    cp_async_commit();
  }
  float2 v[E];
  if (active) {
    const float2* src = p.src + gl * p.src_bstride + (size_t)y * N;
#pragma unroll
    for (int m = 0; m < E; m++) v[m] = src[t + L * m];
  }
  __syncthreads();
  if (active && p.do_inv) warp_fft<N, true, L>(v, buf, tw, t);
  cp_async_wait<0>();
  __syncthreads();  // the staged rows are visible to every warp
  if (active) {
    const float2* us = srow + (size_t)seq * N;
    float* gw = grow + (size_t)seq * N;
#pragma unroll
    for (int m = 0; m < E; m++) {
      const int x = t + L * m;
      const float2 u = us[x];
      gw[x] = p.unit_k * fmaf(v[m].x, u.y, -(v[m].y * u.x));
      const float2 M = staged_mask<PRE>(p, mrow, x, y);
      v[m] = cmul(v[m], make_float2(M.x, -M.y));
    }
  }
  __syncthreads();  // every warp's gradient terms are in shared memory
  {
    const int nf = min(fw, nfields - (int)blockIdx.y * fw);
    float* gp = (blockIdx.y == 0 ? p.grad_dn : p.grad_part + (size_t)(blockIdx.y - 1) * p.grad_part_stride) + zoff +
                (size_t)y * N;
    for (int x = threadIdx.x; x < N; x += T) {
      float sacc = grow[x];
      for (int w = 1; w < nf; w++) sacc += grow[(size_t)w * N + x];
      gp[x] = p.grad_acc ? gp[x] + sacc : sacc;
    }
  }
  if (!active || !p.do_fwd) return;
  warp_fft<N, false, L>(v, buf, tw, t);
  float2* dst = p.W + gl * plane + (size_t)y * N;
#pragma unroll
  for (int m = 0; m < E; m++) dst[t + L * m] = v[m];
}

// Sum of the adjoint's per-block gradient partials: grad += part[1] + part[2] + ... in block
// order (part[0] is grad itself), planes 1 .. nz-1
__global__ void grad_parts_sum_kernel(float* grad, const float* part, long long stride, int nparts, size_t n0,
                                      size_t n) {
  const size_t i = n0 + (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float sacc = grad[i];
  for (int b = 1; b < nparts; b++) sacc += part[(size_t)(b - 1) * stride + i];
  grad[i] = sacc;
}

// Column pass without the tile transposition (128 <= N <= 1024, with or without scattering sums). The
// block's 32*C threads load C columns (16, or 8 or 4 for small non-weighted passes) in the
// coalesced tile mapping — thread (r0, cc) = (tid / C, tid % C) holds rows r0 + 32 i of column
// x0 + cc — and keep that mapping for every pointwise step (the propagator from the
// row-major table or the FP32 recipe, the weighted partial sums, the loads and stores); the
// first and last FFT stages run in it as well (colsplit_first / colsplit_last) and only the
// middle stages per warp, on the column's exchange buffer. WHICH: 0 = forward FFT,
// propagator, inverse FFT; 1 = forward FFT + weighted-mode partial sums (k-space stored back);
// 2 = n from the partial sums, propagator, inverse FFT. The weighted passes keep C = 16: their
// per-block partial sums then group the same elements in the same order as the cluster
// kernel's.
// Column buffers are STRIDE float2 apart: with 16 columns an odd stride puts a half-warp's
// 16 columns on 16 different bank pairs; with 8 columns a half-warp spans two rows of 8
// columns, conflict-free at N = 512 and 1024 for stride BUF + 2, 2-way on some accesses at
// 128 and 256; with 4 columns four rows of 4, conflict-free at 512 and 1024 for BUF + 4
// (BUF is a multiple of 16 there), 2-way at best at 128 and 256 (BUF + 2). Checked for every
// first-stage store and last-stage load of each half-warp by brute force on the CPU.
template <int N, int C = kColWarps, int L = 32>
struct ColSplitCfg {
  static constexpr int BUF = WarpFft<N, L>::BUF;
  static constexpr int STRIDE = C == 4 ? (N / L >= 16 ? BUF + 4 : BUF + 2)
                                       : ((C == 8 && N / L >= 16) ? BUF + 2 : (BUF | 1));
  static constexpr int TW_F2 = (WarpFft<N, L>::TW + 1) & ~1;
  static constexpr int DN_F2 = (TW_F2 + C * STRIDE + 1) & ~1;  // 16-byte aligned
  static constexpr size_t SMEM = (size_t)DN_F2 * sizeof(float2);
  static constexpr size_t SMEM_DN = SMEM + (size_t)16 * N * sizeof(float);  // + dn slice 0 of the tile
  static constexpr size_t SMEM_KY = SMEM + (size_t)N * sizeof(float);       // + the ky^2 column
};

// the propagator on the thread's rows r0 + L i of column x (prop_point's arithmetic): the
// row-major table H (conj(H) for the adjoint; TABLE) or the FP32 recipe with kx^2 of the
// column and the ky^2 table staged in shared memory; with scattering sums
// (bpm_3d.py:335-341) the thread's partials S, G over its rows
template <int N, bool TABLE, bool SCAT, int L>
__device__ __forceinline__ void propagate_rows_t(const ColParams& p, float2 (&v)[N / L], int x, int r0,
                                                 float n_eff, float kx2, const float* sky2, float& S, float& G) {
  const unsigned step = (unsigned)L * (unsigned)p.nx;
  const unsigned off = (unsigned)r0 * (unsigned)p.nx + (unsigned)x;
  const bool cj = p.conj_h;
  const float nkx = TABLE ? 0.f : __fsub_rn(prop_nk(p, n_eff), kx2);
  auto hval = [&](int i) {
    float2 h;
    if constexpr (TABLE) {
      h = __ldg(p.H + off + i * step);
      if (cj) h.y = -h.y;
    } else {
      const float tmp = __fsub_rn(nkx, sky2[r0 + L * i]);
      h = make_float2(0.f, 0.f);
      if (tmp >= 0.f) {
        const float ph = __fmul_rn(-p.dzf, __fsqrt_rn(tmp));
        sincosf(ph, &h.y, &h.x);
      }
    }
    return h;
  };
  if constexpr (!SCAT) {
#pragma unroll
    for (int i = 0; i < N / L; i++) v[i] = cscale(cmul(v[i], hval(i)), p.scale);
    return;
  }
  const float2 plain = (x == 0 && r0 == 0) ? plain_wave(p) : make_float2(0.f, 0.f);
#pragma unroll
  for (int i = 0; i < N / L; i++) {
    const float2 u = cmul(v[i], hval(i));
    float2 d = u;
    if (x == 0 && r0 == 0 && i == 0) d = csub(d, plain);
    const float a2 = cabs2(d);
    S = fmaf(__ldg(p.sw + off + i * step), a2, S);
    G = fmaf(__ldg(p.gw + off + i * step), a2, G);
    v[i] = cscale(u, p.scale);
  }
}
template <int N, bool SCAT, int L>
__device__ __forceinline__ void propagate_rows(const ColParams& p, float2 (&v)[N / L], int x, int r0,
                                               float n_eff, float kx2, const float* sky2, float& S, float& G) {
  if (p.prop_mode == 0)
    propagate_rows_t<N, true, SCAT, L>(p, v, x, r0, n_eff, kx2, sky2, S, G);
  else
    propagate_rows_t<N, false, SCAT, L>(p, v, x, r0, n_eff, kx2, sky2, S, G);
}

// blocks per SM a column kernel of C columns x L threads must fit (registers as row_min_blocks)
__host__ __device__ constexpr int col_min_blocks(int N, int L, int C) {
  return 65536 / ((N / L >= 32 ? 128 : 64) * C * L);
}

template <int N, int WHICH, int C = kColWarps, bool SCAT = false, int L = 32>
__global__ void __launch_bounds__(C * L, col_min_blocks(N, L, C))
col_split_kernel(ColParams p) {
  using Cfg = ColSplitCfg<N, C, L>;
  constexpr int E = N / L;
  constexpr int T = C * L;
  static_assert(C == 16 || ((C == 8 || C == 4) && WHICH == 0), "weighted passes keep 16-column blocks");
  static_assert(!SCAT || (C == 16 && WHICH != 1), "scattering partials per 16-column tile");
  extern __shared__ __align__(16) float2 smem[];
  float2* tw = smem;
  float2* bufs = smem + Cfg::TW_F2;
  __shared__ float red[64];
  __shared__ float s_n;
  const int warp = threadIdx.x >> 5, t = threadIdx.x & 31;
  const int r0 = threadIdx.x / C, cc = threadIdx.x % C;
  const int gl = blockIdx.y;
  const int x0 = blockIdx.x * C;
  float2* Wp = p.W + (size_t)gl * p.nx * N;
  const unsigned gstep = (unsigned)L * (unsigned)p.nx;
  float2* colbuf = bufs + cc * Cfg::STRIDE;                 // column x0 + cc: the tile-mapping stages
  float2* wbuf = bufs + (threadIdx.x / L) * Cfg::STRIDE;    // column x0 + tid/L: the middle stages
  const int wt = threadIdx.x % L;
  // plan constants before the wait for the previous pass: the twiddles, and for the FP32
  // recipe kx^2 of the thread's column and one ky^2 entry per thread (staged after it, in the
  // region the weighted reduction uses for dn)
  constexpr int TWR = (WarpFft<N, L>::TW + T - 1) / T;  // twiddles per thread
  constexpr int KYR = (N + T - 1) / T;                // ky^2 entries per thread
  float2 twv[TWR];
#pragma unroll
  for (int k = 0; k < TWR; k++) {
    const int i = threadIdx.x + k * T;
    twv[k] = i < WarpFft<N, L>::TW ? p.wtw[i] : make_float2(0.f, 0.f);
  }
  const bool recipe = WHICH != 1 && p.prop_mode != 0;
  const float kx2v = recipe ? __ldg(p.kx2 + x0 + cc) : 0.f;
  float kyv[KYR];
#pragma unroll
  for (int k = 0; k < KYR; k++) {
    const int i = threadIdx.x + k * T;
    kyv[k] = (recipe && i < N) ? __ldg(p.ky2 + i) : 0.f;
  }
  float* sky2 = reinterpret_cast<float*>(smem + Cfg::DN_F2);
  dep_wait();
  dep_release();
  // weighted reduction: dn slice 0 of this tile goes to shared memory with cp.async now and
  // is read after the transform; a 16-value row is 2^lg 16-byte pieces
  const char* dn_stage = nullptr;
  if (WHICH == 1 && p.dn && p.dn_stage) {
    const int lg = p.dn_dtype == BPM_DN_F16 ? 1 : 2;
    const int es = 1 << lg;
    char* dst = reinterpret_cast<char*>(smem + Cfg::DN_F2);
    const char* srcb = static_cast<const char*>(p.dn) + ((size_t)gl * p.dn_bstride + x0) * es;
    const size_t rowb = (size_t)p.nx * es;
    for (int ch = threadIdx.x; ch < (N << lg); ch += T)
      cp_async16(dst + (size_t)ch * 16, srcb + (size_t)(ch >> lg) * rowb + (ch & (es - 1)) * 16);
    cp_async_commit();
    dn_stage = dst;
  }
  float2 v[E];
  {
    const unsigned gofs = (unsigned)r0 * (unsigned)p.nx + (unsigned)(x0 + cc);
#pragma unroll
    for (int i = 0; i < E; i++) v[i] = Wp[gofs + i * gstep];
  }
  if (WHICH == 2 && warp == 0) {
    // every block of the field sums the partials in index order, so all get the same n; the
    // lanes fetch them at once (at most 64: nx <= 1024) and pass them on by shuffles
    const int np = p.nx / 16;
    const float* part = p.red_part + (size_t)gl * np * 2;
    const float d0 = t < np ? part[2 * t] : 0.f, u0 = t < np ? part[2 * t + 1] : 0.f;
    const float d1 = t + 32 < np ? part[2 * t + 64] : 0.f, u1 = t + 32 < np ? part[2 * t + 65] : 0.f;
    float dn_sum = 0.f, u_sum = 0.f;
    for (int i = 0; i < np; i++) {
      dn_sum += __shfl_sync(0xffffffffu, i < 32 ? d0 : d1, i & 31);
      u_sum += __shfl_sync(0xffffffffu, i < 32 ? u0 : u1, i & 31);
    }
    if (t == 0) {
      const float dn0 = dn_sum / u_sum;  // mult_dn_mean_buff, bpm_3d_kernels.cl:117
      s_n = p.n00f + dn0;                // mult_propagator_buff, bpm_3d_kernels.cl:482
      if (blockIdx.x == 0) p.dn0_field[gl] = dn0;
    }
  }
#pragma unroll
  for (int k = 0; k < TWR; k++)
    if (threadIdx.x + k * T < WarpFft<N, L>::TW) tw[threadIdx.x + k * T] = twv[k];
#pragma unroll
  for (int k = 0; k < KYR; k++)
    if (recipe && threadIdx.x + k * T < N) sky2[threadIdx.x + k * T] = kyv[k];
  float S = 0.f, G = 0.f;  // scattering partials
  if (WHICH == 2) {
    __syncthreads();  // s_n, ky^2
    propagate_rows<N, SCAT, L>(p, v, x0 + cc, r0, s_n, kx2v, sky2, S, G);
  } else {
    // forward column FFT
    colsplit_first<N, false, L>(v, colbuf, r0);
    __syncthreads();
    colsplit_middle<N, false, L>(wbuf, tw, wt);
    __syncthreads();
    colsplit_last<N, false, L>(v, colbuf, tw, r0);
  }
  if (WHICH == 0) {
    propagate_rows<N, SCAT, L>(p, v, x0 + cc, r0, p.prop_mode == 1 ? p.slice_n[p.z + 1] : p.n00f, kx2v, sky2,
                               S, G);
    __syncthreads();  // every thread has read its last-stage inputs before the buffers are reused
  }
  if (WHICH != 1) {
    if constexpr (SCAT) scat_partials_store<T>(p, S, G, gl, red);
    // inverse column FFT, then the coalesced store
    colsplit_first<N, true, L>(v, colbuf, r0);
    __syncthreads();
    colsplit_middle<N, true, L>(wbuf, tw, wt);
    __syncthreads();
    colsplit_last<N, true, L>(v, colbuf, tw, r0);
    const unsigned gofs = (unsigned)r0 * (unsigned)p.nx + (unsigned)(x0 + cc);
#pragma unroll
    for (int i = 0; i < E; i++) Wp[gofs + i * gstep] = v[i];
  } else {
    // weighted mode: store k-space and sum |u_hat| and |u_hat|*dn over the tile, each thread
    // over its rows in order
    if (dn_stage) cp_async_wait<0>();
    __syncthreads();  // the dn pieces other threads copied
    const unsigned gofs = (unsigned)r0 * (unsigned)p.nx + (unsigned)(x0 + cc);
    float sdn = 0.f, su = 0.f;
    if (dn_stage && p.dn_dtype != BPM_DN_F16) {
      const float* ds = reinterpret_cast<const float*>(dn_stage) + threadIdx.x;
#pragma unroll
      for (int i = 0; i < E; i++) {
        Wp[gofs + i * gstep] = v[i];
        const float a = __fsqrt_rn(cabs2(v[i]));
        su += a;
        sdn = fmaf(a, ds[T * i], sdn);
      }
    } else if (dn_stage) {
      const __half* ds = reinterpret_cast<const __half*>(dn_stage) + threadIdx.x;
#pragma unroll
      for (int i = 0; i < E; i++) {
        Wp[gofs + i * gstep] = v[i];
        const float a = __fsqrt_rn(cabs2(v[i]));
        su += a;
        sdn = fmaf(a, __half2float(ds[T * i]), sdn);
      }
    } else {
#pragma unroll
      for (int i = 0; i < E; i++) {
        const unsigned k = gofs + i * gstep;
        Wp[k] = v[i];
        const float a = __fsqrt_rn(cabs2(v[i]));
        su += a;
        if (p.dn) sdn = fmaf(a, load_dn_real(p.dn, p.dn_dtype, gl * p.dn_bstride + k), sdn);
      }
    }
    block_sum2<T>(sdn, su, red);
    if (threadIdx.x == 0) {
      float* o = p.red_part + ((size_t)gl * (p.nx / 16) + blockIdx.x) * 2;
      o[0] = sdn;
      o[1] = su;
    }
  }
}

// ---------------------------------------------------------------------------------------
// Weighted column pass in one launch (Ny = N in {128, 256, 512}, no scattering sums): the
// plane-wide sums sit between the forward column FFT and the propagator, so the two
// column passes of the weighted mode (col_split_kernel<N, 1> and <N, 2>) become one kernel
// whose blocks of a field form a thread-block cluster. A block is two 16-column tiles side
// by side (two halves of 512 threads, each laid out and computing exactly as one block of
// col_split_kernel: the same FFT stages, the same per-tile partial sums in the same order),
// so a field of nx / 16 tiles is a cluster of nx / 32 blocks (16 at nx = 512). Each half
// stores its tile's two partials in shared memory; after a cluster barrier (a hardware
// barrier over blocks the launch co-schedules: no block waits on a block that has not
// started), one warp per block reads all of the field's partials through distributed
// shared memory in tile order and sums them as col_split_kernel<N, 2> does, so every block
// gets the same n = n0 + dn0 bit for bit. The forward-transformed tile never leaves the
// registers: propagator, inverse FFT and the coalesced store follow directly. A last
// cluster barrier keeps each block's partials alive until every block has read them.
// Results equal the two-pass march bit for bit. Opt-in (bpm_request.col_fuse = 1): a
// cluster of 16 blocks that each fill an SM is placed on few GPCs at a time, and at
// 512 x 512 (8 fields per launch, GB300) the fused pass took 41.2 us against 9.7 + 9.6 us
// for the two passes.
// ---------------------------------------------------------------------------------------
template <int N>
struct FusedCfg {
  using Half = ColSplitCfg<N, kColWarps, 32>;
  static constexpr int T = 2 * kColWarps * 32;                  // 1024 threads: two 16-column tiles
  static constexpr int TW_F2 = Half::TW_F2;
  static constexpr int BUFS_F2 = 2 * kColWarps * Half::STRIDE;  // two halves' column buffers
  static constexpr int DN_F2 = (TW_F2 + BUFS_F2 + 1) & ~1;     // 16-byte aligned
  static constexpr int KY_F = 2 * 16 * N;                       // ky^2 after the two dn tiles (floats)
  static constexpr size_t SMEM = (size_t)DN_F2 * sizeof(float2) + (size_t)(KY_F + N) * sizeof(float);
};

template <int N>
__global__ void __launch_bounds__(FusedCfg<N>::T, 1) col_fused_kernel(ColParams p) {
  using Cfg = FusedCfg<N>;
  using Half = typename Cfg::Half;
  constexpr int L = 32;
  constexpr int E = N / L;
  constexpr int C = kColWarps;  // columns per half
  constexpr int TH = C * L;     // threads per half
  constexpr int T = Cfg::T;
  extern __shared__ __align__(16) float2 smem[];
  __shared__ float red[2][32];
  __shared__ float part[2][2];  // this block's two tile partials (sum |u| dn, sum |u|)
  __shared__ float s_n;
  namespace cg = cooperative_groups;
  cg::cluster_group cl = cg::this_cluster();
  const int h = threadIdx.x / TH, ht = threadIdx.x % TH;
  const int warp = threadIdx.x >> 5, t = threadIdx.x & 31;
  const int r0 = ht / C, cc = ht % C;
  const int gl = blockIdx.y;
  const int x0 = (blockIdx.x * 2 + h) * C;
  float2* tw = smem;
  float2* bufs = smem + Cfg::TW_F2 + h * C * Half::STRIDE;
  float2* Wp = p.W + (size_t)gl * p.nx * N;
  const unsigned gstep = (unsigned)L * (unsigned)p.nx;
  float2* colbuf = bufs + cc * Half::STRIDE;
  float2* wbuf = bufs + (ht / L) * Half::STRIDE;
  const int wt = ht % L;
  float* dnbase = reinterpret_cast<float*>(smem + Cfg::DN_F2);
  float* sky2 = dnbase + Cfg::KY_F;
  // plan constants before the wait for the previous pass: twiddles and ky^2 to shared memory
  for (int i = threadIdx.x; i < WarpFft<N, L>::TW; i += T) tw[i] = p.wtw[i];
  for (int i = threadIdx.x; i < N; i += T) sky2[i] = __ldg(p.ky2 + i);
  dep_wait();
  dep_release();
  const char* dn_stage = nullptr;
  if (p.dn && p.dn_stage) {
    const int lg = p.dn_dtype == BPM_DN_F16 ? 1 : 2;
    const int es = 1 << lg;
    char* dst = reinterpret_cast<char*>(dnbase + h * 16 * N);
    const char* srcb = static_cast<const char*>(p.dn) + ((size_t)gl * p.dn_bstride + x0) * es;
    const size_t rowb = (size_t)p.nx * es;
    for (int ch = ht; ch < (N << lg); ch += TH)
      cp_async16(dst + (size_t)ch * 16, srcb + (size_t)(ch >> lg) * rowb + (ch & (es - 1)) * 16);
    cp_async_commit();
    dn_stage = dst;
  }
  float2 v[E];
  const unsigned gofs = (unsigned)r0 * (unsigned)p.nx + (unsigned)(x0 + cc);
#pragma unroll
  for (int i = 0; i < E; i++) v[i] = Wp[gofs + i * gstep];
  __syncthreads();  // twiddles and ky^2 staged
  // forward column FFT
  colsplit_first<N, false, L>(v, colbuf, r0);
  __syncthreads();
  colsplit_middle<N, false, L>(wbuf, tw, wt);
  __syncthreads();
  colsplit_last<N, false, L>(v, colbuf, tw, r0);
  // the tile's partial sums, each thread over its rows in order, then the half's tree
  if (dn_stage) cp_async_wait<0>();
  __syncthreads();  // the dn pieces other threads copied; every thread is past its last-stage reads
  float sdn = 0.f, su = 0.f;
  if (dn_stage && p.dn_dtype != BPM_DN_F16) {
    const float* ds = reinterpret_cast<const float*>(dn_stage) + ht;
#pragma unroll
    for (int i = 0; i < E; i++) {
      const float a = __fsqrt_rn(cabs2(v[i]));
      su += a;
      sdn = fmaf(a, ds[TH * i], sdn);
    }
  } else if (dn_stage) {
    const __half* ds = reinterpret_cast<const __half*>(dn_stage) + ht;
#pragma unroll
    for (int i = 0; i < E; i++) {
      const float a = __fsqrt_rn(cabs2(v[i]));
      su += a;
      sdn = fmaf(a, __half2float(ds[TH * i]), sdn);
    }
  } else {
#pragma unroll
    for (int i = 0; i < E; i++) {
      const float a = __fsqrt_rn(cabs2(v[i]));
      su += a;
      if (p.dn) sdn = fmaf(a, load_dn_real(p.dn, p.dn_dtype, gl * p.dn_bstride + gofs + i * gstep), sdn);
    }
  }
  // block_sum2<TH> of the half: warp trees, then the half's first thread over its warps in order
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    sdn += __shfl_xor_sync(0xffffffffu, sdn, o);
    su += __shfl_xor_sync(0xffffffffu, su, o);
  }
  const int hw = ht >> 5;
  if (t == 0) {
    red[h][2 * hw] = sdn;
    red[h][2 * hw + 1] = su;
  }
  __syncthreads();
  if (ht == 0) {
    float a = 0.f, b = 0.f;
    for (int i = 0; i < TH / 32; i++) {
      a += red[h][2 * i];
      b += red[h][2 * i + 1];
    }
    part[h][0] = a;
    part[h][1] = b;
  }
  cl.sync();  // every block's tile partials are visible across the cluster
  if (warp == 0) {
    // the field's partials in tile order (tile 2r + k in block rank r, half k), summed as
    // col_split_kernel<N, 2> sums them
    const int np = p.nx / 16;
    float d0 = 0.f, u0 = 0.f, d1 = 0.f, u1 = 0.f;
    if (t < np) {
      const float* pr = cl.map_shared_rank(&part[0][0], t >> 1);
      d0 = pr[2 * (t & 1)];
      u0 = pr[2 * (t & 1) + 1];
    }
    if (t + 32 < np) {
      const float* pr = cl.map_shared_rank(&part[0][0], (t + 32) >> 1);
      d1 = pr[2 * (t & 1)];
      u1 = pr[2 * (t & 1) + 1];
    }
    float dn_sum = 0.f, u_sum = 0.f;
    for (int i = 0; i < np; i++) {
      dn_sum += __shfl_sync(0xffffffffu, i < 32 ? d0 : d1, i & 31);
      u_sum += __shfl_sync(0xffffffffu, i < 32 ? u0 : u1, i & 31);
    }
    if (t == 0) {
      const float dn0 = dn_sum / u_sum;  // mult_dn_mean_buff, bpm_3d_kernels.cl:117
      s_n = p.n00f + dn0;                // mult_propagator_buff, bpm_3d_kernels.cl:482
      if (blockIdx.x == 0) p.dn0_field[gl] = dn0;
    }
  }
  __syncthreads();  // s_n
  float S = 0.f, G = 0.f;
  propagate_rows<N, false, L>(p, v, x0 + cc, r0, s_n, __ldg(p.kx2 + x0 + cc), sky2, S, G);
  // inverse column FFT, then the coalesced store
  colsplit_first<N, true, L>(v, colbuf, r0);
  __syncthreads();
  colsplit_middle<N, true, L>(wbuf, tw, wt);
  __syncthreads();
  colsplit_last<N, true, L>(v, colbuf, tw, r0);
#pragma unroll
  for (int i = 0; i < E; i++) Wp[gofs + i * gstep] = v[i];
  cl.sync();  // no block leaves while another may still read its partials
}

// ---------------------------------------------------------------------------------------
// Whole-march cluster kernel for square grids N = 64, 128, 256: one thread-block cluster of
// C = N/16 blocks per field (16 at 256, a non-portable cluster size) holds the field in
// distributed shared memory for all nz steps. Block c owns rows [16c, 16c+16) (row slab R,
// 16 x N) and columns [16c, 16c+16) (column slab K, N x 17 with one pad column). A step:
// cluster barrier (row slabs ready) -> every block gathers its column slab from the other
// blocks' row slabs through DSMEM (all remote loads of a batch issued before any store) ->
// column FFT, [weighted: per-16-column-tile partial sums, exchanged through DSMEM after a
// cluster barrier], propagator (the block's table columns and ky^2 staged once) -> inverse
// column FFT -> cluster barrier (column slabs ready) -> every block gathers its row slab back
// -> inverse row FFT, phase mask (the next plane's mask rows prefetched by cp.async during
// the column pass), plane output, forward row FFT. The field never leaves the chip; one
// launch runs the whole march of every field of the request. The FFTs, pointwise helpers and
// the weighted partial sums (same 16-column tiles, same 512-thread element order, same
// fixed-order total) are those of the pass kernels, so the results are the same bits (at
// 64, where the pass kernels use the tile FFT, the same to FP32 rounding). Cluster barriers
// are hardware barriers over blocks the launch co-schedules; a final barrier keeps every
// block's shared memory alive until the others have finished reading it.
// ---------------------------------------------------------------------------------------
constexpr int kClusterThreads = 512;  // 16 warps

struct ClusterArgs {
  RowParams rp;
  ColParams cp;
  const float2* u0;  // (batch, N, N)
  int nz;
  int stage_mask;    // the next plane's mask (or dn) rows may be staged with 16-byte cp.async
};

template <int N>
struct ClusterCfg {
  static constexpr int SLAB = 16;                  // rows (and columns) per block
  static constexpr int C = N / SLAB;               // blocks per field (16 at 256: a non-portable size)
  static constexpr int NW = kClusterThreads / 32;
  static constexpr int TWPAD = (WarpFft<N>::TW + 1) & ~1;
  static constexpr int KP = SLAB + 1;              // column-slab row pitch (float2)
  static constexpr int GATHER = N * SLAB / kClusterThreads;  // slab elements per thread
  // the next plane's mask rows and this block's propagator-table columns are staged in
  // shared memory as well
  static constexpr bool STAGE = true;
  static constexpr size_t HT_F2 = STAGE ? (size_t)SLAB * N : 0;
  static constexpr size_t MS_F2 = STAGE ? (size_t)SLAB * N : 0;  // up to 8 bytes per element
  static constexpr size_t F2 = 2 * (size_t)TWPAD + (size_t)SLAB * N + (size_t)N * KP +
                               (size_t)NW * WarpFft<N>::BUF + HT_F2 + MS_F2 + N / 2;
  static constexpr size_t SMEM = F2 * sizeof(float2);
  static_assert(N * SLAB % kClusterThreads == 0 && SLAB % 16 == 0, "slab shape");
};

template <int N>
__global__ void __launch_bounds__(kClusterThreads, 1) cluster_march_kernel(ClusterArgs a) {
  namespace cg = cooperative_groups;
  using Cfg = ClusterCfg<N>;
  constexpr int E = N / 32;
  constexpr int T = kClusterThreads;
  constexpr int NW = Cfg::NW;
  constexpr int SLAB = Cfg::SLAB;
  constexpr int KP = Cfg::KP;
  constexpr int GA = Cfg::GATHER;
  cg::cluster_group cl = cg::this_cluster();
  const int c = (int)cl.block_rank();
  const int gl = blockIdx.x / Cfg::C;
  const RowParams& p = a.rp;
  const ColParams& q = a.cp;
  extern __shared__ __align__(16) float2 csm[];
  float2* twr = csm;
  float2* twc = twr + Cfg::TWPAD;
  float2* R = twc + Cfg::TWPAD;       // SLAB x N
  float2* K = R + SLAB * N;           // N x KP
  float2* X = K + (size_t)N * KP;     // NW exchange buffers
  float2* HT = X + NW * WarpFft<N>::BUF;  // SLAB x N: propagator table columns (STAGE)
  char* MS = reinterpret_cast<char*>(HT + Cfg::HT_F2);  // next plane's mask / dn rows (STAGE)
  float* KY = reinterpret_cast<float*>(HT + Cfg::HT_F2 + Cfg::MS_F2);  // ky^2 (N floats)
  __shared__ float red[64];
  __shared__ float part[2 * (SLAB / 16)];  // this block's tile partials (weighted)
  const int warp = threadIdx.x >> 5, t = threadIdx.x & 31;
  float2* buf = X + warp * WarpFft<N>::BUF;
  for (int k = threadIdx.x; k < WarpFft<N>::TW; k += T) {
    twr[k] = p.wtw[k];
    twc[k] = q.wtw[k];
  }
  for (int k = threadIdx.x; k < N; k += T) KY[k] = q.ky2[k];
  const bool stage_ht = Cfg::STAGE && q.prop_mode == 0;
  if (stage_ht)
    for (int k = threadIdx.x; k < SLAB * N; k += T) HT[k] = q.Ht[(size_t)c * SLAB * N + k];
  const size_t plane = (size_t)N * N;
  const int nz = a.nz;
  const bool stage_mask = Cfg::STAGE && a.stage_mask && p.do_mask;
  const int mes = p.mask ? 8 : (p.dn_dtype == BPM_DN_C64 ? 8 : (p.dn_dtype == BPM_DN_F16 ? 2 : 4));
  float dn0 = 0.f;  // weighted: dn0 of the last column pass

  // the row pass producing plane z over this block's rows (z = 0: plane 0 is the input)
  auto row_phase = [&](int z) {
    const bool first = z == 0;
    // the mean-index shift of plane z (row_dn0 of the pass kernels, whose p.z is the plane)
    float dz0 = 0.f;
    if (!first) {
      if (p.mean_mode == BPM_MEAN_WEIGHTED)
        dz0 = dn0;
      else if (p.mean_mode == BPM_MEAN_SIMPLE && p.slice_dn0)
        dz0 = p.slice_dn0[z];
    }
    const float2 rot = row_rot(p, dz0);
    const size_t zoff = (size_t)z * plane;
    for (int yl = warp; yl < SLAB; yl += NW) {
      const int y = c * SLAB + yl;
      float2 v[E];
      if (first) {
        const float2* src = a.u0 + gl * plane + (size_t)y * N;
#pragma unroll
        for (int m = 0; m < E; m++) v[m] = src[t + 32 * m];
      } else {
#pragma unroll
        for (int m = 0; m < E; m++) v[m] = R[yl * N + t + 32 * m];
        warp_fft<N, true>(v, buf, twr, t);
      }
      const char* mrow = MS + (size_t)yl * N * mes;
#pragma unroll
      for (int m = 0; m < E; m++) {
        const int x = t + 32 * m;
        const size_t pix = (size_t)y * N + x;
        float2 u = v[m];
        if (!first && p.do_mask) {
          float2 M;
          if (stage_mask) {
            if (p.mask)
              M = reinterpret_cast<const float2*>(mrow)[x];
            else if (p.dn_dtype == BPM_DN_C64)
              M = mask_from_complex(reinterpret_cast<const float2*>(mrow)[x], p.unit_k);
            else
              M = mask_from_real(p.dn_dtype == BPM_DN_F16 ? __half2float(reinterpret_cast<const __half*>(mrow)[x])
                                                          : reinterpret_cast<const float*>(mrow)[x],
                                 p.unit_k, x, y, p.nx, p.ny, p.absorb, p.taper);
          } else {
            M = p.mask ? p.mask[zoff + pix]
                       : mask_value(p.dn, p.dn_dtype, gl * p.dn_bstride + zoff + pix, p.unit_k, x, y, p.nx, p.ny,
                                    p.absorb, p.taper);
          }
          u = cmul(u, M);
          if (dz0 != 0.f) u = cmul(u, rot);
        }
        if (p.out_kind == BPM_OUT_FIELD)
          __stcs(reinterpret_cast<float2*>(p.out) + gl * p.out_bstride + zoff + pix, u);
        else if (p.out_kind == BPM_OUT_INTENSITY)
          __stcs(reinterpret_cast<float*>(p.out) + gl * p.out_bstride + zoff + pix, cabs2(u));
        if (z == nz - 1 && p.last_plane) p.last_plane[gl * plane + pix] = u;
        v[m] = u;
      }
      if (z + 1 < nz) {
        warp_fft<N, false>(v, buf, twr, t);
#pragma unroll
        for (int m = 0; m < E; m++) R[yl * N + t + 32 * m] = v[m];
      }
    }
  };

  __syncthreads();  // tables
  row_phase(0);
  for (int i = 0; i + 1 < nz; i++) {
    cl.sync();  // every row slab holds the row-transformed field
    {
      // gather the column slab K[y][xl] = R_{y/SLAB}[y%SLAB][SLAB c + xl]: all remote loads
      // first, then the stores
      float2 g[GA];
#pragma unroll
      for (int k = 0; k < GA; k++) {
        const int e = threadIdx.x + k * T;
        const int y = e / SLAB, xl = e % SLAB;
        const float2* Rr = cl.map_shared_rank(R, y / SLAB);
        g[k] = Rr[(y % SLAB) * N + c * SLAB + xl];
      }
#pragma unroll
      for (int k = 0; k < GA; k++) {
        const int e = threadIdx.x + k * T;
        K[(e / SLAB) * KP + e % SLAB] = g[k];
      }
    }
    if (stage_mask) {
      // the rows of plane i+1's mask (or dn) this block will apply, fetched during the
      // column pass
      const size_t off = (size_t)(i + 1) * plane + (size_t)c * SLAB * N;
      const char* src = p.mask ? reinterpret_cast<const char*>(p.mask + off)
                               : static_cast<const char*>(p.dn) + ((size_t)gl * p.dn_bstride + off) * mes;
      for (int o = threadIdx.x * 16; o < SLAB * N * mes; o += T * 16) cp_async16(MS + o, src + o);
      cp_async_commit();
    }
    __syncthreads();
    float n_eff = q.prop_mode == 1 ? q.slice_n[i + 1] : q.n00f;
    if (q.prop_mode == 2) {
      // weighted: forward transforms, k-space back into the slab, tile partial sums
      for (int xl = warp; xl < SLAB; xl += NW) {
        float2 v[E];
#pragma unroll
        for (int m = 0; m < E; m++) v[m] = K[(t + 32 * m) * KP + xl];
        warp_fft<N, false>(v, buf, twc, t);
#pragma unroll
        for (int m = 0; m < E; m++) K[(t + 32 * m) * KP + xl] = v[m];
      }
      __syncthreads();
      constexpr int PER = 16 * N / T;  // the warp kernels' element order within a tile
      for (int tile = 0; tile < SLAB / 16; tile++) {
        const int x0 = c * SLAB + tile * 16;
        float sdn = 0.f, su = 0.f;
#pragma unroll
        for (int ii = 0; ii < PER; ii++) {
          const int e = threadIdx.x + ii * T;
          const int n = e >> 4, cc = e & 15;
          const float2 u = K[n * KP + tile * 16 + cc];
          const float aa = __fsqrt_rn(cabs2(u));
          su += aa;
          if (q.dn)
            sdn = fmaf(aa, load_dn_real(q.dn, q.dn_dtype, gl * q.dn_bstride + (size_t)n * N + x0 + cc), sdn);
        }
        block_sum2<T>(sdn, su, red);
        if (threadIdx.x == 0) {
          part[2 * tile] = sdn;
          part[2 * tile + 1] = su;
        }
        __syncthreads();
      }
      cl.sync();  // every block's partials are visible
      if (threadIdx.x == 0) {
        float dn_sum = 0.f, u_sum = 0.f;
        for (int r = 0; r < Cfg::C; r++) {
          const float* pr = cl.map_shared_rank(part, r);
          for (int tile = 0; tile < SLAB / 16; tile++) {
            dn_sum += pr[2 * tile];
            u_sum += pr[2 * tile + 1];
          }
        }
        red[0] = dn_sum / u_sum;  // mult_dn_mean_buff, bpm_3d_kernels.cl:117
      }
      __syncthreads();
      dn0 = red[0];
      n_eff = q.n00f + dn0;  // mult_propagator_buff, bpm_3d_kernels.cl:482
    }
    const float nk = prop_nk(q, n_eff);
    for (int xl = warp; xl < SLAB; xl += NW) {
      const int x = c * SLAB + xl;
      float2 v[E];
#pragma unroll
      for (int m = 0; m < E; m++) v[m] = K[(t + 32 * m) * KP + xl];
      if (q.prop_mode != 2) warp_fft<N, false>(v, buf, twc, t);
      float S = 0.f, G = 0.f;
      const float2* htc = stage_ht ? HT + (size_t)xl * N : nullptr;
#pragma unroll
      for (int m = 0; m < E; m++)
        v[m] = prop_point<true>(q, v[m], x, t + 32 * m, nk, make_float2(0.f, 0.f), S, G, KY, htc);
      warp_fft<N, true>(v, buf, twc, t);
#pragma unroll
      for (int m = 0; m < E; m++) K[(t + 32 * m) * KP + xl] = v[m];
    }
    cl.sync();  // every column slab holds the propagated field
    {
      // gather the row slab back: R[yl][x] = K_{x/SLAB}[SLAB c + yl][x%SLAB]
      float2 g[GA];
#pragma unroll
      for (int k = 0; k < GA; k++) {
        const int e = threadIdx.x + k * T;
        const int yl = e / N, x = e % N;
        const float2* Kr = cl.map_shared_rank(K, x / SLAB);
        g[k] = Kr[(c * SLAB + yl) * KP + x % SLAB];
      }
#pragma unroll
      for (int k = 0; k < GA; k++) R[threadIdx.x + k * T] = g[k];
    }
    if (stage_mask) cp_async_wait<0>();  // this thread's pieces of the next plane's mask rows
    __syncthreads();
    row_phase(i + 1);
  }
  cl.sync();  // no block leaves while another may still read its slabs
}

// ---------------------------------------------------------------------------------------
// dispatch over power-of-two sizes
// ---------------------------------------------------------------------------------------
template <template <int> class K>
struct SizeDispatch;

// Row and column kernels for 128 <= N <= 1024: warp-per-row kernels and the
// transposition-free column kernel. A pipelined persistent family (each warp or block
// walking a strided item list and prefetching the next item with cp.async) was measured
// against them on GB300 (512x512x256 weighted, one group of B fields: B = 1 6.3 vs 6.1 ms,
// B = 2 6.6 vs 5.0, B = 8 11.9 vs 7.6; concurrent groups favoured the warp kernels further)
// and removed. Every kernel computes the same bits for a sequence whatever the launch shape
// (explicit fmaf in all shared arithmetic), so a field's result does not depend on the
// batch it marched in.

// 1024-point rows and columns run the warp-FFT kernels (32 values per lane, one exchange
// per transform); BPM_GB300_WARP1024=0 selects the shared-memory tile kernels instead
bool warp1024_enabled() {
  static const bool on = [] {
    const char* e = getenv("BPM_GB300_WARP1024");
    return !(e && strcmp(e, "0") == 0);
  }();
  return on;
}

// SMs of the current device (read once per process)
int sm_count() {
  static const int n = [] {
    int dev = 0, v = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev);
    cudaGetLastError();
    return v > 0 ? v : 1;
  }();
  return n;
}

// blocks of `kernel` resident on the whole device at once
template <class Kern>
int resident_blocks(Kern kernel, int threads, size_t smem) {
  int dev = 0, nsm = 1, occ = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kernel, threads, smem);
  cudaGetLastError();
  return std::max(1, occ) * std::max(1, nsm);
}

// workers for `items` work items with at most `cap` workers, every worker taking the same
// number of items (the last one possibly fewer)
inline int balanced_workers(int items, int cap) {
  const int per = (items + cap - 1) / cap;
  return (items + per - 1) / per;
}

template <int N>
struct RowK {
  static constexpr bool WARP = N >= 128 && N <= 1024;  // sequence-in-registers kernels
  static constexpr bool TILE = !WARP || N == 1024;     // shared-memory tile kernels
  template <int L>
  static void prepare_l() {
    using W = WarpCfg<N, L>;
    cudaFuncSetAttribute(row_adj_shared_kernel<N, 0, L>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)W::adj_smem(kRowWarps));
    cudaFuncSetAttribute(row_adj_shared_kernel<N, 1, L>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)W::adj_smem(kRowWarps));
    cudaFuncSetAttribute(row_shared_kernel<N, 0, L>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)W::ROW_SMEM_SHARED);
    cudaFuncSetAttribute(row_shared_kernel<N, 1, L>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)W::ROW_SMEM_SHARED);
    cudaFuncSetAttribute(row_shared_kernel<N, 0, L, kRowWarps>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)W::ROW_SMEM_SHARED);
    cudaFuncSetAttribute(row_shared_kernel<N, 1, L, kRowWarps>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)W::ROW_SMEM_SHARED);
    cudaFuncSetAttribute(row_warp_kernel<N, false, 0, kRowWarps, L>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)W::ROW_SMEM);
    cudaFuncSetAttribute(row_warp_kernel<N, true, 0, kRowWarps, L>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)W::ROW_SMEM);
    cudaFuncSetAttribute(row_warp_kernel<N, false, 1, kRowWarps, L>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)W::ROW_SMEM);
    cudaFuncSetAttribute(row_warp_kernel<N, true, 1, kRowWarps, L>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)W::ROW_SMEM);
  }
  static void prepare() {
    static PerDevice once;
    once.get([] {
      if constexpr (WARP) {
        prepare_l<32>();
      }
      if constexpr (TILE) {
        cudaFuncSetAttribute(row_pass_kernel<N, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)TileCfg<N>::SMEM);
        cudaFuncSetAttribute(row_pass_kernel<N, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)TileCfg<N>::SMEM);
      }
      return 1;
    });
  }
  // all fields of the group share the slice-z mask row: the precomputed mask, or one dn
  // volume (dn_batch_stride 0, or a group of one field); the row is staged with 16-byte
  // cp.async
  static bool shared_ok(const RowParams& p, int nfields) {
    if (!p.do_mask) return false;
    if (p.mask) return aligned16(p.mask);
    return (p.dn_bstride == 0 || nfields == 1) && aligned16(p.dn);
  }
  // g.x counts 16-row tiles
  static int launch(dim3 g, cudaStream_t s, const RowParams& p, bool adj) {
    prepare();
    if constexpr (WARP) {
      if (N <= 512 || warp1024_enabled()) {
        return launch_warp<32>(g, s, p, adj);
      }
    }
    if constexpr (TILE) {
      if (adj)
        BPM_CUDA_TRY(launch_dep(row_pass_kernel<N, true>, g, dim3(TileCfg<N>::THREADS), TileCfg<N>::SMEM, s, p));
      else
        BPM_CUDA_TRY(launch_dep(row_pass_kernel<N, false>, g, dim3(TileCfg<N>::THREADS), TileCfg<N>::SMEM, s, p));
      BPM_LAUNCH_CHECK("row_pass_kernel");
      return BPM_OK;
    }
    set_error("row pass: no kernel for this size");
    return BPM_ERR_SHAPE;
  }
  template <int L>
  static int launch_warp(dim3 g, cudaStream_t s, const RowParams& p, bool adj) {
    if constexpr (WARP) {
      constexpr int BUF = WarpFft<N, L>::BUF;
      // a single field takes this kernel too (one-warp blocks): its mask or dn row is staged
      // by cp.async at block start, so the row's DRAM read overlaps the inverse row FFT
      // instead of following it as in row_warp_kernel (GB300, one field, Nz 128, same bits:
      // 1024^2 ignore 3.63 -> 2.55 ms, 512^2 2.04 -> 1.14 ms, 512^2 weighted 3.00 -> 2.05 ms)
      if (adj && p.grad_sum && p.do_mask && p.z > 0 && (p.mask ? aligned16(p.mask) : aligned16(p.dn))) {
        // the dn gradient summed over the group's fields, a block per row and up to 8 fields
        const int nb = ((int)g.y + kRowWarps - 1) / kRowWarps;
        const int fw = ((int)g.y + nb - 1) / nb;
        const int threads = (fw * L + 31) / 32 * 32;
        const size_t sm = WarpCfg<N, L>::adj_smem(threads / L);
        auto fn = p.mask ? row_adj_shared_kernel<N, 1, L> : row_adj_shared_kernel<N, 0, L>;
        BPM_CUDA_TRY(launch_dep(fn, dim3(p.ny, nb), dim3(threads), sm, s, p, (int)g.y, fw));
        BPM_LAUNCH_CHECK("row_adj_shared_kernel");
        return BPM_OK;
      }
      if (!adj && shared_ok(p, (int)g.y)) {
        // fields per block: the group split evenly over ceil(G / 8) blocks per row
        const int nb = ((int)g.y + kRowWarps - 1) / kRowWarps;
        const int fw = ((int)g.y + nb - 1) / nb;
        const int threads = (fw * L + 31) / 32 * 32;
        const size_t sm = ((size_t)2 * N + (size_t)(threads / L) * BUF) * sizeof(float2);
        auto fn = fw == kRowWarps ? (p.mask ? row_shared_kernel<N, 1, L, kRowWarps> : row_shared_kernel<N, 0, L, kRowWarps>)
                                  : (p.mask ? row_shared_kernel<N, 1, L> : row_shared_kernel<N, 0, L>);
        BPM_CUDA_TRY(launch_dep(fn, dim3(p.ny, nb), dim3(threads), sm, s, p, (int)g.y, fw));
        BPM_LAUNCH_CHECK("row_shared_kernel");
        return BPM_OK;
      }
      // with fewer 8-row blocks than twice the SMs (a single field's adjoint or unaligned
      // mask, small per-field-dn groups), blocks of 2 rows spread the pass over 4 times as
      // many SMs
      const int rows = (int)(g.x * 16) * (int)g.y;
      if (rows / kRowWarps < 2 * sm_count()) {
        const dim3 gw(g.x * 16 / 2, g.y);
        auto fn = adj ? (p.mask ? row_warp_kernel<N, true, 1, 2, L> : row_warp_kernel<N, true, 0, 2, L>)
                      : (p.mask ? row_warp_kernel<N, false, 1, 2, L> : row_warp_kernel<N, false, 0, 2, L>);
        BPM_CUDA_TRY(launch_dep(fn, gw, dim3(2 * L), WarpCfg<N, L>::row_smem(2), s, p));
        BPM_LAUNCH_CHECK("row_warp_kernel");
        return BPM_OK;
      }
      const dim3 gw(g.x * 16 / kRowWarps, g.y);
      auto fn = adj ? (p.mask ? row_warp_kernel<N, true, 1, kRowWarps, L> : row_warp_kernel<N, true, 0, kRowWarps, L>)
                    : (p.mask ? row_warp_kernel<N, false, 1, kRowWarps, L> : row_warp_kernel<N, false, 0, kRowWarps, L>);
      BPM_CUDA_TRY(launch_dep(fn, gw, dim3(kRowWarps * L), WarpCfg<N, L>::ROW_SMEM, s, p));
      BPM_LAUNCH_CHECK("row_warp_kernel");
      return BPM_OK;
    }
    return BPM_ERR_SHAPE;
  }
};

template <int N, int WHICH>
struct ColK {
  static constexpr bool SPLIT = N >= 128 && N <= 1024;  // col_split_kernel
  static constexpr bool TILE = !SPLIT || N == 1024;     // shared-memory tile kernels
  static void (*fn())(ColParams) {
    if constexpr (TILE)
      return WHICH == 0 ? col_pass_kernel<N> : (WHICH == 1 ? col_fwd_reduce_kernel<N> : col_inv_kernel<N>);
    return nullptr;
  }
  static constexpr int threads() { return TileCfg<N>::THREADS; }
  static constexpr size_t smem() { return TileCfg<N>::SMEM; }
  template <int L>
  static constexpr size_t split_smem() {
    return WHICH == 1 ? ColSplitCfg<N, kColWarps, L>::SMEM_DN : ColSplitCfg<N, kColWarps, L>::SMEM_KY;
  }
  template <int L>
  static constexpr size_t split8_smem() { return ColSplitCfg<N, 8, L>::SMEM_KY; }
  template <int L>
  static constexpr size_t split4_smem() { return ColSplitCfg<N, 4, L>::SMEM_KY; }
  template <int L>
  static void prepare_l() {
    cudaFuncSetAttribute(col_split_kernel<N, WHICH, kColWarps, false, L>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)split_smem<L>());
    if constexpr (WHICH == 0) {
      cudaFuncSetAttribute(col_split_kernel<N, 0, 8, false, L>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)split8_smem<L>());
      cudaFuncSetAttribute(col_split_kernel<N, 0, 4, false, L>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)split4_smem<L>());
    }
    if constexpr (WHICH != 1)
      cudaFuncSetAttribute(col_split_kernel<N, WHICH, kColWarps, true, L>,
                           cudaFuncAttributeMaxDynamicSharedMemorySize, (int)split_smem<L>());
  }
  static void prepare() {
    static PerDevice once;
    once.get([] {
      if constexpr (TILE) cudaFuncSetAttribute(fn(), cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem());
      if constexpr (SPLIT) prepare_l<32>();
      return 1;
    });
  }
  template <int L>
  static int launch_split(dim3 g, cudaStream_t s, const ColParams& p) {
    // a non-weighted pass with fewer 16-column blocks than SMs runs 8-column blocks, so twice
    // as many SMs share it (the columns' arithmetic is the same); so does every non-weighted
    // pass with 32 values per thread, whose 16-column blocks take half an SM's registers; and
    // with fewer 8-column blocks than SMs and up to 16 values per thread (a single field of
    // 256 or 512 rows), 4-column blocks (GB300, one field, Nz 128: 512^2 ignore 1.12 -> 1.03
    // ms, 256^2 0.68 -> 0.62 ms; at 1024 rows they measured slower, 2.53 -> 2.94 ms)
    if constexpr (WHICH == 0) {
      const bool quarter =
          p.col_block == 4 || (p.col_block == 0 && N / L < 32 && (int)(g.x * 2 * g.y) < sm_count());
      if (!p.scat && quarter) {
        BPM_CUDA_TRY(launch_dep(col_split_kernel<N, 0, 4, false, L>, dim3(g.x * 4, g.y), dim3(4 * L),
                                split4_smem<L>(), s, p));
        BPM_LAUNCH_CHECK("col_split_kernel");
        return BPM_OK;
      }
      const bool narrow = p.col_block == 8 || (p.col_block == 0 && ((int)(g.x * g.y) < sm_count() || N / L >= 32));
      if (!p.scat && narrow) {
        BPM_CUDA_TRY(launch_dep(col_split_kernel<N, 0, 8, false, L>, dim3(g.x * 2, g.y), dim3(8 * L),
                                split8_smem<L>(), s, p));
        BPM_LAUNCH_CHECK("col_split_kernel");
        return BPM_OK;
      }
    }
    if constexpr (WHICH != 1) {
      if (p.scat) {
        BPM_CUDA_TRY(launch_dep(col_split_kernel<N, WHICH, kColWarps, true, L>, g, dim3(kColWarps * L),
                                split_smem<L>(), s, p));
        BPM_LAUNCH_CHECK("col_split_kernel");
        return BPM_OK;
      }
    }
    BPM_CUDA_TRY(launch_dep(col_split_kernel<N, WHICH, kColWarps, false, L>, g, dim3(kColWarps * L),
                            split_smem<L>(), s, p));
    BPM_LAUNCH_CHECK("col_split_kernel");
    return BPM_OK;
  }
  static int launch(dim3 g, cudaStream_t s, const ColParams& p) {
    prepare();
    if constexpr (SPLIT) {
      if (N <= 512 || warp1024_enabled()) {
        return launch_split<32>(g, s, p);
      }
    }
    if constexpr (TILE) {
      BPM_CUDA_TRY(launch_dep(fn(), g, dim3(threads()), smem(), s, p));
      BPM_LAUNCH_CHECK("col_pass_kernel");
      return BPM_OK;
    }
    set_error("column pass: no kernel for this size");
    return BPM_ERR_SHAPE;
  }
};

// The fused weighted column pass (col_fused_kernel<N>): a cluster of nx / 32 blocks per
// field. state: -1 not checked yet, 0 this cluster size cannot be launched here, 1 ready
template <int N>
struct FusedK {
  static PerDevice& state(int cl) {
    static PerDevice st[17];
    return st[cl];
  }
  static cudaLaunchConfig_t config(dim3 g, int cl, cudaStream_t s, cudaLaunchAttribute* at, bool pdl) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = g;
    cfg.blockDim = dim3(FusedCfg<N>::T);
    cfg.dynamicSmemBytes = FusedCfg<N>::SMEM;
    cfg.stream = s;
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = cl;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    at[1].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[1].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = pdl ? 2 : 1;
    return cfg;
  }
  // the kernel fits and clusters of `cl` blocks can be co-scheduled on this device
  static bool ready(int cl) {
    return state(cl).get([cl] {
      int ok = 0;
      if (cl > 8) cudaFuncSetAttribute(col_fused_kernel<N>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
      if (cudaFuncSetAttribute(col_fused_kernel<N>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)FusedCfg<N>::SMEM) == cudaSuccess) {
        cudaLaunchAttribute at[2];
        cudaLaunchConfig_t cfg = config(dim3(cl, 1), cl, nullptr, at, false);
        int clusters = 0;
        if (cudaOccupancyMaxActiveClusters(&clusters, col_fused_kernel<N>, &cfg) == cudaSuccess) ok = clusters > 0;
      }
      cudaGetLastError();
      return ok;
    }) == 1;
  }
  static int launch(dim3 g, int cl, cudaStream_t s, const ColParams& p) {
    cudaLaunchAttribute at[2];
    cudaLaunchConfig_t cfg = config(g, cl, s, at, true);
    BPM_CUDA_TRY(cudaLaunchKernelEx(&cfg, col_fused_kernel<N>, p));
    BPM_LAUNCH_CHECK("col_fused_kernel");
    return BPM_OK;
  }
};

int launch_row(int N, dim3 g, cudaStream_t s, const RowParams& p, bool adj = false) {
  switch (N) {
    case 16: return RowK<16>::launch(g, s, p, adj);
    case 32: return RowK<32>::launch(g, s, p, adj);
    case 64: return RowK<64>::launch(g, s, p, adj);
    case 128: return RowK<128>::launch(g, s, p, adj);
    case 256: return RowK<256>::launch(g, s, p, adj);
    case 512: return RowK<512>::launch(g, s, p, adj);
    case 1024: return RowK<1024>::launch(g, s, p, adj);
  }
  set_error("unsupported nx");
  return BPM_ERR_SHAPE;
}

template <int WHICH>
int launch_col(int N, dim3 g, cudaStream_t s, const ColParams& p) {
  switch (N) {
    case 16: return ColK<16, WHICH>::launch(g, s, p);
    case 32: return ColK<32, WHICH>::launch(g, s, p);
    case 64: return ColK<64, WHICH>::launch(g, s, p);
    case 128: return ColK<128, WHICH>::launch(g, s, p);
    case 256: return ColK<256, WHICH>::launch(g, s, p);
    case 512: return ColK<512, WHICH>::launch(g, s, p);
    case 1024: return ColK<1024, WHICH>::launch(g, s, p);
  }
  set_error("unsupported ny");
  return BPM_ERR_SHAPE;
}

// raise the dynamic shared-memory limit of every kernel a plan will launch (outside any
// stream capture)
template <int N>
void prepare_size() {
  RowK<N>::prepare();
  ColK<N, 0>::prepare();
  ColK<N, 1>::prepare();
  ColK<N, 2>::prepare();
}

void prepare_kernels(int nx, int ny) {
  for (int n : {nx, ny}) {
    switch (n) {
      case 16: prepare_size<16>(); break;
      case 32: prepare_size<32>(); break;
      case 64: prepare_size<64>(); break;
      case 128: prepare_size<128>(); break;
      case 256: prepare_size<256>(); break;
      case 512: prepare_size<512>(); break;
      case 1024: prepare_size<1024>(); break;
    }
  }
}

int default_group(const bpm_plan* pl, int batch) {
  const size_t plane_bytes = (size_t)pl->d.nx * pl->d.ny * 8;
  // up to kMaxConcurrentGroups groups march at once: keep each group's planes near 16 MB so
  // all of them stay resident in the 129 MB L2 next to the dn slices and output streams
  const int g = (int)std::max<size_t>(1, (16u << 20) / plane_bytes);
  return std::max(1, std::min(g, batch));
}

struct WsLayout {
  size_t w, red, dn0, scat, total;
};

WsLayout ws_layout(const bpm_plan* pl, int G) {
  WsLayout L;
  const int ntiles = pl->d.nx / 16;
  size_t off = 0;
  L.w = off;
  off += align256((size_t)G * pl->d.nx * pl->d.ny * sizeof(float2));
  L.red = off;
  off += align256((size_t)G * ntiles * 2 * sizeof(float));
  L.dn0 = off;
  off += align256((size_t)G * sizeof(float));
  L.scat = off;
  off += align256((size_t)G * ntiles * 2 * sizeof(float));
  L.total = off;
  return L;
}

int check_request(const bpm_plan* pl, const bpm_request* r) {
  if (!r) { set_error("request is NULL"); return BPM_ERR_ARG; }
  if (r->batch < 1) { set_error("batch must be >= 1"); return BPM_ERR_ARG; }
  if (!r->u0) { set_error("u0 is NULL"); return BPM_ERR_ARG; }
  if (r->dn_dtype < BPM_DN_NONE || r->dn_dtype > BPM_DN_C64) { set_error("bad dn_dtype"); return BPM_ERR_ARG; }
  if (r->dn_dtype != BPM_DN_NONE && !r->dn) { set_error("dn is NULL but dn_dtype is set"); return BPM_ERR_ARG; }
  if (r->dn_dtype == BPM_DN_C64 && pl->d.mean_mode != BPM_MEAN_IGNORE) {
    set_error("complex dn is only defined for mean_mode='ignore'");
    return BPM_ERR_UNSUPPORTED;
  }
  if (pl->d.mean_mode == BPM_MEAN_SIMPLE && (!r->slice_n || !r->slice_dn0)) {
    set_error("mean_mode='simple' needs slice_n and slice_dn0");
    return BPM_ERR_ARG;
  }
  if (r->out_kind < BPM_OUT_NONE || r->out_kind > BPM_OUT_INTENSITY) { set_error("bad out_kind"); return BPM_ERR_ARG; }
  if (r->out_kind != BPM_OUT_NONE && !r->out) { set_error("out is NULL but out_kind is set"); return BPM_ERR_ARG; }
  if (r->scatter_g && !r->scatter_p) { set_error("scatter_g needs scatter_p"); return BPM_ERR_ARG; }
  if (r->group < 0) { set_error("group must be >= 0"); return BPM_ERR_ARG; }
  if (r->conc < 0 || r->conc > kMaxConcurrentGroups) { set_error("conc must be in 0..8"); return BPM_ERR_ARG; }
  if (r->col_block != 0 && r->col_block != 4 && r->col_block != 8 && r->col_block != 16) {
    set_error("col_block must be 0, 4, 8 or 16");
    return BPM_ERR_ARG;
  }
  if (r->cluster < 0 || r->cluster > 2) { set_error("cluster must be 0, 1 or 2"); return BPM_ERR_ARG; }
  if (r->col_fuse < 0 || r->col_fuse > 2) { set_error("col_fuse must be 0, 1 or 2"); return BPM_ERR_ARG; }
  if (r->ckpt && r->ckpt_every < 1) { set_error("ckpt_every must be >= 1 with ckpt"); return BPM_ERR_ARG; }
  if (r->mask && (r->dn_dtype == BPM_DN_NONE || r->dn_batch_stride != 0 || ((uintptr_t)r->mask & 7))) {
    set_error("mask needs one shared dn volume and 8-byte alignment");
    return BPM_ERR_ARG;
  }
  if (r->ckpt && ((uintptr_t)r->ckpt & 15)) { set_error("ckpt must be 16-byte aligned"); return BPM_ERR_ARG; }
  // 16-byte alignment of the vectorised accesses
  auto mis = [](const void* q) { return ((uintptr_t)q & 15) != 0; };
  if (mis(r->u0) || (r->out && mis(r->out)) || (r->last_plane && mis(r->last_plane))) {
    set_error("u0/out/last_plane must be 16-byte aligned");
    return BPM_ERR_ARG;
  }
  if (r->dn && (mis(r->dn) || (r->dn_batch_stride & 1))) {
    set_error("dn must be 16-byte aligned with an even dn_batch_stride");
    return BPM_ERR_ARG;
  }
  return BPM_OK;
}

// launch parameters of one group of fields [b0, b0+Gc) of a request
struct MarchCtx {
  RowParams rp;
  ColParams cp;
  dim3 grow, gcol;
};

int group_size(const bpm_plan* pl, const bpm_request* r) {
  return r->group > 0 ? std::min(r->group, r->batch) : default_group(pl, r->batch);
}

int check_workspace(const bpm_plan* pl, const bpm_request* r, const void* ws, size_t ws_bytes) {
  WsLayout L = ws_layout(pl, group_size(pl, r));
  if (!ws || ws_bytes < L.total) {
    set_error("workspace too small: need " + std::to_string(L.total) + " bytes");
    return BPM_ERR_OOM;
  }
  if ((uintptr_t)ws & 15) {
    set_error("workspace must be 16-byte aligned");
    return BPM_ERR_ARG;
  }
  return BPM_OK;
}

MarchCtx make_ctx(const bpm_plan* pl, const bpm_request* r, void* ws, int b0, int Gc) {
  const bpm_grid_desc& d = pl->d;
  const int nx = d.nx, ny = d.ny, nz = d.nz;
  WsLayout L = ws_layout(pl, group_size(pl, r));
  char* wsb = static_cast<char*>(ws);
  float2* W = reinterpret_cast<float2*>(wsb + L.w);
  float* red = reinterpret_cast<float*>(wsb + L.red);
  float* dn0f = reinterpret_cast<float*>(wsb + L.dn0);
  float* scatp = reinterpret_cast<float*>(wsb + L.scat);
  const size_t plane = (size_t)nx * ny;
  const bool has_dn = r->dn_dtype != BPM_DN_NONE;
  const size_t dn_esize = r->dn_dtype == BPM_DN_C64 ? 8 : (r->dn_dtype == BPM_DN_F16 ? 2 : 4);
  const size_t out_esize = r->out_kind == BPM_OUT_FIELD ? 8 : 4;

  MarchCtx c;
  RowParams& rp = c.rp;
  memset(&rp, 0, sizeof(rp));
  rp.W = W;
  rp.nx = nx; rp.ny = ny; rp.nz = nz;
  rp.dn = has_dn ? static_cast<const char*>(r->dn) + (size_t)b0 * r->dn_batch_stride * dn_esize : nullptr;
  rp.dn_dtype = r->dn_dtype;
  rp.dn_bstride = r->dn_batch_stride;
  rp.unit_k = pl->unit_k;
  rp.absorb = d.absorbing_width;
  rp.taper = pl->taper;
  rp.mean_mode = d.mean_mode;
  rp.dn0_field = dn0f;
  rp.slice_dn0 = r->slice_dn0;
  rp.out = r->out ? static_cast<char*>(r->out) + (size_t)b0 * r->out_batch_stride * out_esize : nullptr;
  rp.out_kind = r->out ? r->out_kind : BPM_OUT_NONE;
  rp.out_bstride = r->out_batch_stride;
  rp.last_plane = r->last_plane ? static_cast<float2*>(r->last_plane) + (size_t)b0 * plane : nullptr;
  rp.scat_part = scatp;
  rp.n_ctiles = nx / 16;
  rp.scat_p = r->scatter_p ? r->scatter_p + (size_t)b0 * nz : nullptr;
  rp.scat_g = r->scatter_g ? r->scatter_g + (size_t)b0 * nz : nullptr;
  rp.prefac_f = (float)(1. / nx / ny * d.dx * d.dy);
  rp.tw = pl->tw_x;
  rp.wtw = pl->wtw_x;
  rp.src = W;
  rp.src_bstride = plane;
  rp.zout0 = 0;
  rp.mask = static_cast<const float2*>(r->mask);
  if (r->ckpt) {
    rp.ckpt_every = r->ckpt_every;
    rp.n_ckpt = (nz - 1) / r->ckpt_every + 1;
    rp.ckpt = static_cast<float2*>(r->ckpt) + (size_t)b0 * rp.n_ckpt * plane;
  }

  ColParams& cp = c.cp;
  memset(&cp, 0, sizeof(cp));
  cp.W = W;
  cp.nx = nx; cp.ny = ny; cp.nz = nz;
  cp.prop_mode = d.mean_mode == BPM_MEAN_IGNORE ? 0 : (d.mean_mode == BPM_MEAN_SIMPLE ? 1 : 2);
  cp.H = pl->H;
  cp.Ht = pl->Ht;
  cp.kx2 = pl->kx2;
  cp.ky2 = pl->ky2;
  cp.k0f = pl->k0f;
  cp.dzf = pl->dzf;
  cp.n00f = pl->n0f;
  cp.slice_n = r->slice_n;
  cp.scale = 1.f / (float)plane;
  cp.dn = rp.dn;
  cp.dn_dtype = r->dn_dtype;
  cp.dn_bstride = r->dn_batch_stride;
  cp.red_part = red;
  cp.dn0_field = dn0f;
  cp.scat = r->scatter_p != nullptr;
  cp.sw = pl->sw;
  cp.gw = pl->gw;
  cp.scat_part = scatp;
  cp.plain_phase = pl->k0 * d.n0 * d.dz;
  cp.spi = r->scattering_plane_ind;
  cp.tw = pl->tw_y;
  cp.wtw = pl->wtw_y;
  {
    const int es = r->dn_dtype == BPM_DN_F16 ? 2 : 4;
    cp.dn_stage = (r->dn_dtype == BPM_DN_F32 || r->dn_dtype == BPM_DN_F16) && cp.dn && aligned16(cp.dn) &&
                  ((size_t)r->dn_batch_stride * es) % 16 == 0 && ((size_t)nx * es) % 16 == 0;
  }

  cp.col_block = r->col_block;
  cp.col_fuse = r->col_fuse;
  c.grow = dim3(ny / 16, Gc);
  c.gcol = dim3(nx / 16, Gc);
  return c;
}

// the first row pass: plane 0 is the input itself, then the forward row FFT of step 0
int launch_first_row(const bpm_plan* pl, const bpm_request* r, MarchCtx& c, int b0, cudaStream_t s) {
  RowParams rp = c.rp;
  rp.src = static_cast<const float2*>(r->u0) + (size_t)b0 * pl->d.nx * pl->d.ny;
  rp.z = 0;
  rp.do_inv = 0;
  rp.do_fwd = pl->d.nz > 1;
  rp.do_mask = 0;
  return launch_row(pl->d.nx, c.grow, s, rp);
}

// kNoFused when the fused column pass does not serve this request, else its launch status
constexpr int kNoFused = 1;
int try_fused_cols(const bpm_plan* pl, const MarchCtx& c, cudaStream_t s, bool force) {
  const ColParams& p = c.cp;
  const int nx = pl->d.nx, ny = pl->d.ny;
  if (pl->d.mean_mode != BPM_MEAN_WEIGHTED || p.scat || (!force && p.col_fuse != 1) || nx % 32 || nx / 32 > 16)
    return kNoFused;
  const int cl = nx / 32;
  const dim3 g(cl, c.gcol.y);
  switch (ny) {
    case 128: return FusedK<128>::ready(cl) ? FusedK<128>::launch(g, cl, s, p) : kNoFused;
    case 256: return FusedK<256>::ready(cl) ? FusedK<256>::launch(g, cl, s, p) : kNoFused;
    case 512: return FusedK<512>::ready(cl) ? FusedK<512>::launch(g, cl, s, p) : kNoFused;
  }
  return kNoFused;
}

// the column pass(es) of step i (plane i -> plane i+1): which = 0 the whole step (the fused
// weighted pass where the request asks for it), 1 / 2 the weighted mode's first / second
// pass, 3 the fused weighted pass
int launch_cols(const bpm_plan* pl, MarchCtx& c, int i, int which, cudaStream_t s) {
  c.cp.z = i;
  if (pl->d.mean_mode == BPM_MEAN_WEIGHTED) {
    if (which == 0 || which == 3) {
      const int rc = try_fused_cols(pl, c, s, which == 3);
      if (rc != kNoFused) return rc;
      if (which == 3) {
        set_error("the fused weighted column pass does not serve this grid or request");
        return BPM_ERR_UNSUPPORTED;
      }
    }
    if (which != 2) {
      int rc = launch_col<1>(pl->d.ny, c.gcol, s, c.cp);
      if (rc || which == 1) return rc;
    }
    return launch_col<2>(pl->d.ny, c.gcol, s, c.cp);
  }
  return launch_col<0>(pl->d.ny, c.gcol, s, c.cp);
}

// the row pass producing plane z >= 1
int launch_row_z(const bpm_plan* pl, const bpm_request* r, MarchCtx& c, int z, cudaStream_t s) {
  RowParams rp = c.rp;
  rp.z = z;
  rp.do_inv = 1;
  rp.do_fwd = (z + 1 < pl->d.nz);
  rp.do_mask = r->dn_dtype != BPM_DN_NONE;
  return launch_row(pl->d.nx, c.grow, s, rp);
}

// Destination of bpm_propagate_to_host: the output volume is also copied, run of `chunk`
// planes by run of `chunk` planes, to host memory laid out like req->out.
struct HostSink {
  char* host;
  int chunk;
};

// After the group's stream s has produced planes [z0, z1) of fields [b0, b0+Gc), the
// copy stream moves them to the host: one strided copy (a row per field) when the batch
// stride fits the copy engine's pitch limit, else one copy per field.
int sink_copy(bpm_plan* pl, const bpm_request* r, const HostSink& h, int b0, int Gc, int z0, int z1,
              cudaStream_t s, cudaEvent_t ev) {
  const size_t es = r->out_kind == BPM_OUT_FIELD ? 8 : 4;
  const size_t plane = (size_t)pl->d.nx * pl->d.ny;
  const size_t pitch = (size_t)r->out_batch_stride * es;
  const size_t off = (size_t)b0 * pitch + (size_t)z0 * plane * es;
  const size_t width = (size_t)(z1 - z0) * plane * es;
  const char* src = static_cast<const char*>(r->out) + off;
  BPM_CUDA_TRY(cudaEventRecord(ev, s));
  BPM_CUDA_TRY(cudaStreamWaitEvent(pl->copy, ev, 0));
  if (Gc == 1 || pitch <= (size_t)pl->max_pitch) {
    BPM_CUDA_TRY(cudaMemcpy2DAsync(h.host + off, pitch, src, pitch, width, Gc, cudaMemcpyDeviceToHost, pl->copy));
  } else {
    for (int g = 0; g < Gc; g++)
      BPM_CUDA_TRY(cudaMemcpyAsync(h.host + off + g * pitch, src + g * pitch, width, cudaMemcpyDeviceToHost,
                                   pl->copy));
  }
  return BPM_OK;
}

// The whole-march cluster kernel serves square grids without scattering sums or
// checkpoints. Measured on GB300, one field: at 64^2 it beats the pass kernels (Nz 64
// weighted 0.40 vs 0.82 ms); at 128^2 the pass kernels are faster since a single field's row
// pass stages its mask row (Nz 128 weighted 1.08 vs 1.14 ms, ignore 0.59 vs 0.81 ms, the
// same bits), and at 256^2 too (Nz 256 ignore 1.47 vs 2.70 ms). So by default it takes
// N = 64; BPM_GB300_CLUSTER=1 extends it to 128 and 256, =0 turns it off, and a side
// length (64, 128 or 256) makes it the default up to that side.
bool cluster_enabled(int n) {
  static const int max_side = [] {
    const char* e = getenv("BPM_GB300_CLUSTER");
    if (!e) return 64;
    if (strcmp(e, "0") == 0) return 0;
    if (strcmp(e, "1") == 0) return 256;
    const int v = atoi(e);
    return v >= 64 ? v : 64;
  }();
  return n <= max_side;
}

template <int N>
struct ClusterK {
  static cudaLaunchConfig_t config(unsigned batch, cudaStream_t s, cudaLaunchAttribute* at) {
    using Cfg = ClusterCfg<N>;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(batch * Cfg::C);
    cfg.blockDim = dim3(kClusterThreads);
    cfg.dynamicSmemBytes = Cfg::SMEM;
    cfg.stream = s;
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = Cfg::C;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    return cfg;
  }
  // per device: 0 = no cluster of this shape fits, 1 = launchable
  static bool ready() {
    static PerDevice state;
    return state.get([] {
      int ok = 0;
      if (ClusterCfg<N>::C > 8)
        cudaFuncSetAttribute(cluster_march_kernel<N>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
      if (cudaFuncSetAttribute(cluster_march_kernel<N>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)ClusterCfg<N>::SMEM) == cudaSuccess) {
        cudaLaunchAttribute at[1];
        cudaLaunchConfig_t cfg = config(1, nullptr, at);
        int clusters = 0;
        if (cudaOccupancyMaxActiveClusters(&clusters, cluster_march_kernel<N>, &cfg) == cudaSuccess)
          ok = clusters > 0;
      }
      cudaGetLastError();
      return ok;
    }) == 1;
  }
  static int launch(const bpm_plan* pl, const bpm_request* r, void* ws, cudaStream_t s) {
    MarchCtx c = make_ctx(pl, r, ws, 0, r->batch);
    ClusterArgs a;
    a.rp = c.rp;
    a.rp.do_mask = r->dn_dtype != BPM_DN_NONE;
    a.cp = c.cp;
    a.u0 = static_cast<const float2*>(r->u0);
    a.nz = pl->d.nz;
    {
      const int es = r->mask ? 8 : (r->dn_dtype == BPM_DN_C64 ? 8 : (r->dn_dtype == BPM_DN_F16 ? 2 : 4));
      a.stage_mask = r->mask ? aligned16(r->mask)
                             : (aligned16(r->dn) && ((size_t)r->dn_batch_stride * es) % 16 == 0);
    }
    cudaLaunchAttribute at[1];
    cudaLaunchConfig_t cfg = config((unsigned)r->batch, s, at);
    BPM_CUDA_TRY(cudaLaunchKernelEx(&cfg, cluster_march_kernel<N>, a));
    BPM_LAUNCH_CHECK("cluster_march_kernel");
    return BPM_OK;
  }
};

// kNotCluster when the request is not for the cluster kernel, else its launch status
constexpr int kNotCluster = 1;
int try_cluster_march(const bpm_plan* pl, const bpm_request* r, void* ws, cudaStream_t s) {
  const bpm_grid_desc& d = pl->d;
  const bool want = r->cluster == 1 || (r->cluster == 0 && cluster_enabled(d.nx));
  if (d.nx != d.ny || !want || r->scatter_p || r->ckpt || !pl->wtw_x || !pl->wtw_y) return kNotCluster;
  switch (d.nx) {
    case 64: return ClusterK<64>::ready() ? ClusterK<64>::launch(pl, r, ws, s) : kNotCluster;
    case 128: return ClusterK<128>::ready() ? ClusterK<128>::launch(pl, r, ws, s) : kNotCluster;
    case 256: return ClusterK<256>::ready() ? ClusterK<256>::launch(pl, r, ws, s) : kNotCluster;
  }
  return kNotCluster;
}

// All groups of a request. With room for several workspace slots, groups march
// concurrently on the plan's auxiliary streams (forked from and joined back to s through
// events, which also captures into a CUDA graph as parallel branches), so one group's
// kernels fill the device while another's run their tail waves; otherwise they march one
// after the other on s. Groups marching at the same time are enqueued step by step in
// turn, so work (and, with a host sink, the finished planes handed to the copy stream)
// reaches the device in the order it can run.
int enqueue_march(bpm_plan* pl, const bpm_request* r, void* ws, size_t ws_bytes, cudaStream_t s,
                  const HostSink* sink = nullptr) {
  int rc = check_workspace(pl, r, ws, ws_bytes);
  if (rc) return rc;
  const int nz = pl->d.nz;
  {
    const int crc = try_cluster_march(pl, r, ws, s);
    if (crc != kNotCluster) {
      if (crc != BPM_OK) return crc;
      if (sink) {
        if ((rc = sink_copy(pl, r, *sink, 0, r->batch, 0, nz, s, pl->ev_ready[0]))) return rc;
        BPM_CUDA_TRY(cudaEventRecord(pl->ev_copied, pl->copy));
        BPM_CUDA_TRY(cudaStreamWaitEvent(s, pl->ev_copied, 0));
      }
      return BPM_OK;
    }
  }
  const int G = group_size(pl, r);
  const int ngroups = (r->batch + G - 1) / G;
  const size_t slot = ws_layout(pl, G).total;
  const int conc = std::max(
      1, (int)std::min<size_t>({(size_t)ngroups, ws_bytes / slot, (size_t)(r->conc > 0 ? r->conc : conc_limit())}));
  cudaStream_t st[kMaxConcurrentGroups];
  for (int j = 0; j < conc; j++) st[j] = conc > 1 ? pl->aux[j] : s;
  if (conc > 1 || sink) BPM_CUDA_TRY(cudaEventRecord(pl->ev_fork, s));
  if (conc > 1)
    for (int j = 0; j < conc; j++) BPM_CUDA_TRY(cudaStreamWaitEvent(st[j], pl->ev_fork, 0));
  if (sink) BPM_CUDA_TRY(cudaStreamWaitEvent(pl->copy, pl->ev_fork, 0));
  for (int w0 = 0; w0 < ngroups; w0 += conc) {
    const int nwave = std::min(conc, ngroups - w0);
    MarchCtx c[kMaxConcurrentGroups];
    int b0[kMaxConcurrentGroups], Gc[kMaxConcurrentGroups], zdone[kMaxConcurrentGroups];
    for (int j = 0; j < nwave; j++) {
      b0[j] = (w0 + j) * G;
      Gc[j] = std::min(G, r->batch - b0[j]);
      zdone[j] = 0;
      c[j] = make_ctx(pl, r, static_cast<char*>(ws) + (size_t)j * slot, b0[j], Gc[j]);
      if ((rc = launch_first_row(pl, r, c[j], b0[j], st[j]))) return rc;
    }
    for (int i = 0; i + 1 < nz || (i == 0 && nz == 1); i++) {
      for (int j = 0; j < nwave; j++) {
        if (i + 1 < nz) {
          if ((rc = launch_cols(pl, c[j], i, 0, st[j]))) return rc;
          if ((rc = launch_row_z(pl, r, c[j], i + 1, st[j]))) return rc;
        }
        const int z1 = std::min(i + 2, nz);  // planes [0, z1) of the group are written
        if (sink) {
          // a group's first run goes out after 2 planes, so the host link, the slower side,
          // starts early; later runs are sink->chunk planes
          const int run = zdone[j] == 0 ? std::min(sink->chunk, 2) : sink->chunk;
          if ((z1 - zdone[j] >= run || z1 == nz) && z1 > zdone[j]) {
            if ((rc = sink_copy(pl, r, *sink, b0[j], Gc[j], zdone[j], z1, st[j], pl->ev_ready[j]))) return rc;
            zdone[j] = z1;
          }
        }
      }
    }
  }
  if (conc > 1) {
    for (int j = 0; j < conc; j++) {
      BPM_CUDA_TRY(cudaEventRecord(pl->ev_join[j], st[j]));
      BPM_CUDA_TRY(cudaStreamWaitEvent(s, pl->ev_join[j], 0));
    }
  }
  if (sink) {
    BPM_CUDA_TRY(cudaEventRecord(pl->ev_copied, pl->copy));
    BPM_CUDA_TRY(cudaStreamWaitEvent(s, pl->ev_copied, 0));
  }
  return BPM_OK;
}

// ---------------------------------------------------------------------------------------
// adjoint march
// ---------------------------------------------------------------------------------------
struct BwLayout {
  size_t fwd, adj, seg, part, total;
};

// gradient partial volumes of a summed-gradient adjoint (grad_sum): one per row block past
// the first, ceil(G / 8) blocks per row
inline int bw_grad_parts(int G) { return (G + kRowWarps - 1) / kRowWarps - 1; }

BwLayout bw_layout(const bpm_plan* pl, int G, int k) {
  BwLayout L;
  const size_t plane = (size_t)pl->d.nx * pl->d.ny;
  size_t off = 0;
  L.fwd = off;
  off += ws_layout(pl, G).total;
  L.adj = off;
  off += ws_layout(pl, G).total;
  L.seg = off;
  off += align256((size_t)G * (k + 1) * plane * sizeof(float2));
  L.part = off;
  off += align256((size_t)bw_grad_parts(G) * pl->d.nz * plane * sizeof(float));
  L.total = off;
  return L;
}

int check_backward(const bpm_plan* pl, const bpm_request* r, const void* grad_last, const float* grad_dn) {
  if (pl->d.mean_mode != BPM_MEAN_IGNORE) {
    set_error("the adjoint is defined for mean_mode='ignore' (the propagator must not depend on dn)");
    return BPM_ERR_UNSUPPORTED;
  }
  if (r->dn_dtype == BPM_DN_C64) {
    set_error("the adjoint needs real dn");
    return BPM_ERR_UNSUPPORTED;
  }
  if (!r->ckpt || r->ckpt_every < 1) {
    set_error("the adjoint needs the forward checkpoints (req->ckpt, req->ckpt_every)");
    return BPM_ERR_ARG;
  }
  if (!grad_last || ((uintptr_t)grad_last & 15)) { set_error("grad_last must be a 16-byte aligned pointer"); return BPM_ERR_ARG; }
  if (r->dn_dtype != BPM_DN_NONE && (!grad_dn || ((uintptr_t)grad_dn & 15))) {
    set_error("grad_dn must be a 16-byte aligned pointer");
    return BPM_ERR_ARG;
  }
  if (r->grad_sum != 0 && r->grad_sum != 1) { set_error("grad_sum must be 0 or 1"); return BPM_ERR_ARG; }
  if (r->grad_sum && (r->dn_dtype == BPM_DN_NONE || r->dn_batch_stride != 0)) {
    set_error("grad_sum needs one dn volume shared by the fields (dn_batch_stride 0)");
    return BPM_ERR_ARG;
  }
  // the summed gradient comes from row_adj_shared_kernel: warp-FFT rows, staged 16-byte rows
  if (r->grad_sum && (pl->d.nx < 128 || pl->d.nx > 1024 || (pl->d.nx == 1024 && !warp1024_enabled()) ||
                      !aligned16(r->dn) || (r->mask && !aligned16(r->mask)))) {
    set_error("grad_sum needs 128 <= nx <= 1024 (warp-FFT rows) and 16-byte aligned dn and mask");
    return BPM_ERR_ARG;
  }
  return BPM_OK;
}

int enqueue_backward(bpm_plan* pl, const bpm_request* r, const void* grad_last, float* grad_dn, void* grad_u0,
                     void* ws, size_t ws_bytes, cudaStream_t s) {
  const bpm_grid_desc& d = pl->d;
  const int nz = d.nz, k = r->ckpt_every;
  const int G = group_size(pl, r);
  BwLayout L = bw_layout(pl, G, k);
  if (!ws || ws_bytes < L.total || ((uintptr_t)ws & 15)) {
    set_error("workspace too small or misaligned: need " + std::to_string(L.total) + " bytes");
    return BPM_ERR_OOM;
  }
  char* wsb = static_cast<char*>(ws);
  const size_t plane = (size_t)d.nx * d.ny;
  const int n_ckpt = (nz - 1) / k + 1;
  const int nseg = (nz - 1 + k - 1) / k;  // segments (s*k, min(s*k+k, nz-1)]
  float2* seg = reinterpret_cast<float2*>(wsb + L.seg);
  float* part = reinterpret_cast<float*>(wsb + L.part);
  const bool gsum = r->grad_sum && grad_dn;
  int rc;
  for (int b0 = 0; b0 < r->batch; b0 += G) {
    const int Gc = std::min(G, r->batch - b0);
    // forward recompute context on its own workspace, writing fields into the segment buffer
    MarchCtx cf = make_ctx(pl, r, wsb + L.fwd, b0, Gc);
    cf.rp.out = seg;
    cf.rp.out_kind = BPM_OUT_FIELD;
    cf.rp.out_bstride = (long long)(k + 1) * plane;
    cf.rp.last_plane = nullptr;
    cf.rp.ckpt = nullptr;
    cf.rp.scat_p = cf.rp.scat_g = nullptr;
    cf.cp.scat = 0;
    // adjoint context
    MarchCtx ca = make_ctx(pl, r, wsb + L.adj, b0, Gc);
    ca.rp.out = nullptr;
    ca.rp.out_kind = BPM_OUT_NONE;
    ca.rp.last_plane = nullptr;
    ca.rp.ckpt = nullptr;
    ca.rp.scat_p = ca.rp.scat_g = nullptr;
    ca.rp.seg = seg;
    ca.rp.seg_bstride = (long long)(k + 1) * plane;
    ca.rp.grad_dn = grad_dn ? (gsum ? grad_dn : grad_dn + (size_t)b0 * nz * plane) : nullptr;
    ca.rp.grad_sum = gsum ? 1 : 0;
    ca.rp.grad_part = part;
    ca.rp.grad_part_stride = (long long)nz * plane;
    ca.rp.grad_acc = b0 > 0 ? 1 : 0;
    ca.rp.grad_u0 = grad_u0 ? static_cast<float2*>(grad_u0) + (size_t)b0 * plane : nullptr;
    ca.cp.scat = 0;
    ca.cp.conj_h = 1;
    const float2* ck = static_cast<const float2*>(r->ckpt) + (size_t)b0 * n_ckpt * plane;
    const float2* gl = static_cast<const float2*>(grad_last) + (size_t)b0 * plane;
    for (int sgi = nseg - 1; sgi >= 0; sgi--) {
      const int zs = sgi * k, ze = std::min(zs + k, nz - 1);
      // recompute planes zs..ze of the forward march from checkpoint sgi
      RowParams rp = cf.rp;
      rp.src = ck + (size_t)sgi * plane;
      rp.src_bstride = (long long)n_ckpt * plane;
      rp.z = zs;
      rp.zout0 = zs;
      rp.do_inv = 0;
      rp.do_fwd = 1;
      rp.do_mask = 0;
      if ((rc = launch_row(d.nx, cf.grow, s, rp))) return rc;
      for (int i = zs; i < ze; i++) {
        cf.cp.z = i;
        if ((rc = launch_col<0>(d.ny, cf.gcol, s, cf.cp))) return rc;
        rp = cf.rp;
        rp.z = i + 1;
        rp.zout0 = zs;
        rp.do_inv = 1;
        rp.do_fwd = (i + 1 < ze);
        rp.do_mask = r->dn_dtype != BPM_DN_NONE;
        if ((rc = launch_row(d.nx, cf.grow, s, rp))) return rc;
      }
      // march the adjoint from plane ze down to plane zs
      for (int z = ze; z > zs; z--) {
        RowParams ra = ca.rp;
        ra.z = z;
        ra.seg_z0 = zs;
        ra.do_mask = r->dn_dtype != BPM_DN_NONE;
        ra.do_fwd = 1;
        if (z == nz - 1) {
          ra.src = gl;
          ra.src_bstride = plane;
          ra.do_inv = 0;
        } else {
          ra.do_inv = 1;
        }
        if ((rc = launch_row(d.nx, ca.grow, s, ra, true))) return rc;
        ca.cp.z = z - 1;
        if ((rc = launch_col<0>(d.ny, ca.gcol, s, ca.cp))) return rc;
      }
    }
    // plane 0: the adjoint there is the u0 gradient
    RowParams ra = ca.rp;
    ra.z = 0;
    ra.do_mask = 0;
    ra.do_fwd = 0;
    if (nz == 1) {
      ra.src = gl;
      ra.src_bstride = plane;
      ra.do_inv = 0;
    } else {
      ra.do_inv = 1;
    }
    if ((rc = launch_row(d.nx, ca.grow, s, ra, true))) return rc;
  }
  const int nparts = bw_grad_parts(G) + 1;
  if (gsum && nparts > 1 && nz > 1) {
    // the row blocks' partial sums, added in block order (planes 1 .. nz-1)
    const size_t n0 = plane, n = (size_t)nz * plane;
    grad_parts_sum_kernel<<<(unsigned)((n - n0 + 255) / 256), 256, 0, s>>>(grad_dn, part, (long long)nz * plane,
                                                                           nparts, n0, n);
    BPM_LAUNCH_CHECK("grad_parts_sum_kernel");
  }
  return BPM_OK;
}

}  // namespace

// ---------------------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------------------
extern "C" int bpm_grid_check(const bpm_grid_desc* d) {
  clear_error();
  if (!d) { set_error("grid description is NULL"); return BPM_ERR_ARG; }
  if (!is_pow2(d->nx) || !is_pow2(d->ny) || d->nx < 16 || d->ny < 16 || d->nx > 1024 || d->ny > 1024) {
    set_error("nx and ny must be powers of two in [16, 1024] (got " + std::to_string(d->nx) + ", " +
              std::to_string(d->ny) + ")");
    return BPM_ERR_SHAPE;
  }
  if (d->nz < 1) { set_error("nz must be >= 1"); return BPM_ERR_SHAPE; }
  if (!(d->dx > 0) || !(d->dy > 0) || !(d->dz > 0)) { set_error("units must be positive"); return BPM_ERR_ARG; }
  if (!(d->lam > 0)) { set_error("lam must be positive"); return BPM_ERR_ARG; }
  if (!(d->n0 > 0)) { set_error("n0 must be positive"); return BPM_ERR_ARG; }
  if (d->absorbing_width < 0) { set_error("absorbing_width must be >= 0"); return BPM_ERR_ARG; }
  if (d->mean_mode < BPM_MEAN_IGNORE || d->mean_mode > BPM_MEAN_WEIGHTED) {
    set_error("mean_mode unknown");
    return BPM_ERR_SHAPE;
  }
  if (d->prop_kind != BPM_PROP_FUNCTIONAL && d->prop_kind != BPM_PROP_CLASS) {
    set_error("prop_kind unknown");
    return BPM_ERR_ARG;
  }
  return BPM_OK;
}

// the plan's own streams and events (no device synchronisation)
static cudaError_t create_plan_streams(bpm_plan* pl) {
  cudaError_t e;
  for (int i = 0; i < kMaxConcurrentGroups; i++) {
    if ((e = cudaStreamCreateWithFlags(&pl->aux[i], cudaStreamNonBlocking))) return e;
    if ((e = cudaEventCreateWithFlags(&pl->ev_join[i], cudaEventDisableTiming))) return e;
    if ((e = cudaEventCreateWithFlags(&pl->ev_ready[i], cudaEventDisableTiming))) return e;
  }
  if ((e = cudaEventCreateWithFlags(&pl->ev_fork, cudaEventDisableTiming))) return e;
  if ((e = cudaStreamCreateWithFlags(&pl->copy, cudaStreamNonBlocking))) return e;
  return cudaEventCreateWithFlags(&pl->ev_copied, cudaEventDisableTiming);
}

extern "C" int bpm_plan_create(const bpm_grid_desc* d, bpm_plan** out) {
  int rc = bpm_grid_check(d);
  if (rc) return rc;
  if (!out) { set_error("out is NULL"); return BPM_ERR_ARG; }
  *out = nullptr;
  bpm_plan* pl = new bpm_plan();
  memset(pl, 0, sizeof(*pl));
  pl->d = *d;
  pl->owns_tables = true;
  const int nx = d->nx, ny = d->ny;
  pl->k0 = 2. * M_PI / d->lam;
  pl->k0f = (float)pl->k0;
  pl->dzf = (float)d->dz;
  pl->n0f = (float)d->n0;
  pl->unit_k = (float)(pl->k0 * d->dz);
  cudaGetDevice(&pl->device);

  std::vector<float2> twx(nx), twy(ny);
  for (int k = 0; k < nx; k++) {
    double a = -2. * M_PI * k / nx;
    twx[k] = make_float2((float)cos(a), (float)sin(a));
  }
  for (int k = 0; k < ny; k++) {
    double a = -2. * M_PI * k / ny;
    twy[k] = make_float2((float)cos(a), (float)sin(a));
  }
  std::vector<float> kx2(nx), ky2(ny);
  const float twopi_f = 2.f * PI_F;
  for (int i = 0; i < nx; i++) {
    float k = twopi_f * fftfreq_f32(i, nx, (float)d->dx);
    kx2[i] = k * k;
  }
  for (int j = 0; j < ny; j++) {
    float k = twopi_f * fftfreq_f32(j, ny, (float)d->dy);
    ky2[j] = k * k;
  }
  const int aw = d->absorbing_width;
  std::vector<float> taper(std::max(aw, 1), 1.f);
  for (int i = 0; i < aw; i++) taper[i] = taper_value(i, aw);

  auto fail = [&](cudaError_t e, const char* what) {
    int r = cuda_fail(e, what);
    bpm_plan_destroy(pl);
    return r;
  };
  cudaError_t e;
  if ((e = cudaMalloc(&pl->tw_x, nx * sizeof(float2)))) return fail(e, "cudaMalloc");
  if ((e = cudaMalloc(&pl->tw_y, ny * sizeof(float2)))) return fail(e, "cudaMalloc");
  if ((e = cudaMalloc(&pl->kx2, nx * sizeof(float)))) return fail(e, "cudaMalloc");
  if ((e = cudaMalloc(&pl->ky2, ny * sizeof(float)))) return fail(e, "cudaMalloc");
  if ((e = cudaMalloc(&pl->taper, taper.size() * sizeof(float)))) return fail(e, "cudaMalloc");
  if ((e = cudaMalloc(&pl->H, (size_t)nx * ny * sizeof(float2)))) return fail(e, "cudaMalloc");
  if ((e = cudaMalloc(&pl->Ht, (size_t)nx * ny * sizeof(float2)))) return fail(e, "cudaMalloc");
  if ((e = cudaMalloc(&pl->sw, (size_t)nx * ny * sizeof(float)))) return fail(e, "cudaMalloc");
  if ((e = cudaMalloc(&pl->gw, (size_t)nx * ny * sizeof(float)))) return fail(e, "cudaMalloc");
  if ((e = cudaMemcpy(pl->tw_x, twx.data(), nx * sizeof(float2), cudaMemcpyHostToDevice))) return fail(e, "cudaMemcpy");
  if ((e = cudaMemcpy(pl->tw_y, twy.data(), ny * sizeof(float2), cudaMemcpyHostToDevice))) return fail(e, "cudaMemcpy");
  if ((e = cudaMemcpy(pl->kx2, kx2.data(), nx * sizeof(float), cudaMemcpyHostToDevice))) return fail(e, "cudaMemcpy");
  if ((e = cudaMemcpy(pl->ky2, ky2.data(), ny * sizeof(float), cudaMemcpyHostToDevice))) return fail(e, "cudaMemcpy");
  if ((e = cudaMemcpy(pl->taper, taper.data(), taper.size() * sizeof(float), cudaMemcpyHostToDevice)))
    return fail(e, "cudaMemcpy");
  for (int axis = 0; axis < 2; axis++) {
    const int n = axis == 0 ? nx : ny;
    if (n < 64 || n > 1024) continue;  // the warp FFT's sizes (the cluster kernel uses 64 too)
    std::vector<float2> w = warp_twiddles(n);
    float2** dst = axis == 0 ? &pl->wtw_x : &pl->wtw_y;
    if ((e = cudaMalloc(dst, w.size() * sizeof(float2)))) return fail(e, "cudaMalloc");
    if ((e = cudaMemcpy(*dst, w.data(), w.size() * sizeof(float2), cudaMemcpyHostToDevice)))
      return fail(e, "cudaMemcpy");
  }
  dim3 tb(128), tg((nx + 127) / 128, ny);
  build_tables_kernel<<<tg, tb>>>(nx, ny, d->dx, d->dy, d->dz, d->n0, pl->k0, pl->n0f, pl->k0f, d->prop_kind,
                                  d->use_fresnel_approx, pl->kx2, pl->ky2, pl->H, pl->Ht, pl->sw, pl->gw);
  if ((e = cudaGetLastError())) return fail(e, "build_tables_kernel");
  count_launch();
  if ((e = cudaDeviceSynchronize())) return fail(e, "build_tables_kernel");
  prepare_kernels(nx, ny);
  if ((e = create_plan_streams(pl))) return fail(e, "stream/event creation");
  if ((e = cudaDeviceGetAttribute(&pl->max_pitch, cudaDevAttrMaxPitch, pl->device))) return fail(e, "cudaDeviceGetAttribute");
  *out = pl;
  return BPM_OK;
}

extern "C" int bpm_plan_derive(const bpm_plan* base, int nz, bpm_plan** out) {
  clear_error();
  if (!base || !out) { set_error("base or out is NULL"); return BPM_ERR_ARG; }
  *out = nullptr;
  bpm_grid_desc d = base->d;
  d.nz = nz;
  int rc = bpm_grid_check(&d);
  if (rc) return rc;
  bpm_plan* pl = new bpm_plan(*base);  // the same device tables, read only
  pl->d = d;
  pl->owns_tables = false;
  for (int i = 0; i < kMaxConcurrentGroups; i++) pl->aux[i] = nullptr, pl->ev_join[i] = pl->ev_ready[i] = nullptr;
  pl->ev_fork = pl->ev_copied = nullptr;
  pl->copy = nullptr;
  cudaError_t e = create_plan_streams(pl);
  if (e) {
    bpm_plan_destroy(pl);
    return cuda_fail(e, "stream/event creation");
  }
  *out = pl;
  return BPM_OK;
}

extern "C" int bpm_plan_destroy(bpm_plan* pl) {
  if (!pl) return BPM_OK;
  if (pl->owns_tables) {
    cudaFree(pl->tw_x);
    cudaFree(pl->tw_y);
    cudaFree(pl->wtw_x);
    cudaFree(pl->wtw_y);
    cudaFree(pl->kx2);
    cudaFree(pl->ky2);
    cudaFree(pl->taper);
    cudaFree(pl->H);
    cudaFree(pl->Ht);
    cudaFree(pl->sw);
    cudaFree(pl->gw);
  }
  for (int i = 0; i < kMaxConcurrentGroups; i++) {
    if (pl->aux[i]) cudaStreamDestroy(pl->aux[i]);
    if (pl->ev_join[i]) cudaEventDestroy(pl->ev_join[i]);
    if (pl->ev_ready[i]) cudaEventDestroy(pl->ev_ready[i]);
  }
  if (pl->ev_fork) cudaEventDestroy(pl->ev_fork);
  if (pl->copy) cudaStreamDestroy(pl->copy);
  if (pl->ev_copied) cudaEventDestroy(pl->ev_copied);
  delete pl;
  return BPM_OK;
}

extern "C" int bpm_group_size(const bpm_plan* pl, int batch, int group) {
  if (!pl || batch < 1 || group < 0) return 0;
  return group > 0 ? std::min(group, batch) : default_group(pl, batch);
}

extern "C" size_t bpm_workspace_bytes_conc(const bpm_plan* pl, int batch, int group, int conc) {
  if (!pl || batch < 1 || conc < 0 || conc > kMaxConcurrentGroups) return 0;
  const int G = group > 0 ? std::min(group, batch) : default_group(pl, batch);
  const int ngroups = (batch + G - 1) / G;
  return (size_t)std::min(ngroups, conc > 0 ? conc : conc_limit()) * ws_layout(pl, G).total;
}

extern "C" size_t bpm_workspace_bytes(const bpm_plan* pl, int batch, int group) {
  return bpm_workspace_bytes_conc(pl, batch, group, 0);
}

extern "C" int bpm_propagate(bpm_plan* pl, const bpm_request* r, void* ws, size_t ws_bytes, void* stream) {
  clear_error();
  if (!pl) { set_error("plan is NULL"); return BPM_ERR_ARG; }
  int rc = check_request(pl, r);
  if (rc) return rc;
  return enqueue_march(pl, r, ws, ws_bytes, static_cast<cudaStream_t>(stream));
}

extern "C" int bpm_propagate_to_host(bpm_plan* pl, const bpm_request* r, void* host_out, int chunk_planes,
                                     void* ws, size_t ws_bytes, void* stream) {
  clear_error();
  if (!pl) { set_error("plan is NULL"); return BPM_ERR_ARG; }
  int rc = check_request(pl, r);
  if (rc) return rc;
  if (!host_out || !r->out || r->out_kind == BPM_OUT_NONE) {
    set_error("bpm_propagate_to_host needs host_out and a device output volume (out, out_kind)");
    return BPM_ERR_ARG;
  }
  if (chunk_planes < 1) { set_error("chunk_planes must be >= 1"); return BPM_ERR_ARG; }
  if (r->out_batch_stride < (long long)pl->d.nz * pl->d.nx * pl->d.ny) {
    set_error("out_batch_stride must hold nz planes");
    return BPM_ERR_ARG;
  }
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, r->out) != cudaSuccess || a.type != cudaMemoryTypeDevice) {
    cudaGetLastError();
    set_error("out must be device memory for bpm_propagate_to_host");
    return BPM_ERR_ARG;
  }
  HostSink h{static_cast<char*>(host_out), chunk_planes};
  return enqueue_march(pl, r, ws, ws_bytes, static_cast<cudaStream_t>(stream), &h);
}

extern "C" int bpm_launch_pass(bpm_plan* pl, const bpm_request* r, void* ws, size_t ws_bytes, int pass, int z,
                               void* stream) {
  clear_error();
  if (!pl) { set_error("plan is NULL"); return BPM_ERR_ARG; }
  int rc = check_request(pl, r);
  if (rc) return rc;
  if ((rc = check_workspace(pl, r, ws, ws_bytes))) return rc;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const int Gc = group_size(pl, r);
  MarchCtx c = make_ctx(pl, r, ws, 0, Gc);
  switch (pass) {
    case BPM_PASS_FIRST_ROW:
      return launch_first_row(pl, r, c, 0, s);
    case BPM_PASS_COLUMN:
    case BPM_PASS_COLUMN_REDUCE:
    case BPM_PASS_COLUMN_PROPAGATE:
    case BPM_PASS_COLUMN_FUSED: {
      if (z < 0 || z + 1 >= pl->d.nz) { set_error("column pass needs 0 <= z < nz-1"); return BPM_ERR_ARG; }
      const bool w = pl->d.mean_mode == BPM_MEAN_WEIGHTED;
      if (w == (pass == BPM_PASS_COLUMN)) { set_error("pass kind does not match the mean mode"); return BPM_ERR_ARG; }
      const int which = pass == BPM_PASS_COLUMN ? 0
                        : pass == BPM_PASS_COLUMN_REDUCE ? 1
                        : pass == BPM_PASS_COLUMN_PROPAGATE ? 2 : 3;
      return launch_cols(pl, c, z, which, s);
    }
    case BPM_PASS_ROW:
      if (z < 1 || z >= pl->d.nz) { set_error("row pass needs 1 <= z < nz"); return BPM_ERR_ARG; }
      return launch_row_z(pl, r, c, z, s);
  }
  set_error("unknown pass kind");
  return BPM_ERR_ARG;
}

extern "C" size_t bpm_backward_workspace_bytes(const bpm_plan* pl, int batch, int group, int ckpt_every) {
  if (!pl || batch < 1 || ckpt_every < 1) return 0;
  const int G = group > 0 ? std::min(group, batch) : default_group(pl, batch);
  return bw_layout(pl, G, ckpt_every).total;
}

extern "C" int bpm_backward(bpm_plan* pl, const bpm_request* r, const void* grad_last, float* grad_dn,
                            void* grad_u0, void* ws, size_t ws_bytes, void* stream) {
  clear_error();
  if (!pl) { set_error("plan is NULL"); return BPM_ERR_ARG; }
  int rc = check_request(pl, r);
  if (rc) return rc;
  if ((rc = check_backward(pl, r, grad_last, grad_dn))) return rc;
  if (grad_u0 && ((uintptr_t)grad_u0 & 15)) { set_error("grad_u0 must be 16-byte aligned"); return BPM_ERR_ARG; }
  return enqueue_backward(pl, r, grad_last, grad_dn, grad_u0, ws, ws_bytes, static_cast<cudaStream_t>(stream));
}

extern "C" int bpm_mask_precompute(bpm_plan* pl, const void* dn, int dn_dtype, void* mask, void* stream) {
  clear_error();
  if (!pl || !dn || !mask) { set_error("plan, dn and mask must be given"); return BPM_ERR_ARG; }
  if (dn_dtype != BPM_DN_F32 && dn_dtype != BPM_DN_F16 && dn_dtype != BPM_DN_C64) {
    set_error("bad dn_dtype");
    return BPM_ERR_ARG;
  }
  if (((uintptr_t)mask & 7) || ((uintptr_t)dn & 7)) { set_error("dn and mask must be 8-byte aligned"); return BPM_ERR_ARG; }
  const bpm_grid_desc& d = pl->d;
  dim3 g((d.nx + 127) / 128, d.ny, d.nz);
  mask_precompute_kernel<<<g, 128, 0, static_cast<cudaStream_t>(stream)>>>(
      dn, dn_dtype, pl->unit_k, d.nx, d.ny, d.absorbing_width, pl->taper, static_cast<float2*>(mask));
  BPM_LAUNCH_CHECK("mask_precompute_kernel");
  return BPM_OK;
}

extern "C" int bpm_exec_create(bpm_plan* pl, const bpm_request* r, void* ws, size_t ws_bytes, bpm_exec** out) {
  clear_error();
  if (!pl || !out) { set_error("plan/out is NULL"); return BPM_ERR_ARG; }
  int rc = check_request(pl, r);
  if (rc) return rc;
  cudaStream_t s;
  BPM_CUDA_TRY(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
  unsigned long long before = g_launches.load();
  cudaError_t e = cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal);
  if (e) {
    cudaStreamDestroy(s);
    return cuda_fail(e, "cudaStreamBeginCapture");
  }
  rc = enqueue_march(pl, r, ws, ws_bytes, s);
  cudaGraph_t g = nullptr;
  e = cudaStreamEndCapture(s, &g);
  cudaStreamDestroy(s);
  // captured launches do not run now: take them back off the counter
  unsigned long long n = g_launches.load() - before;
  g_launches.fetch_sub(n);
  if (rc) {
    if (g) cudaGraphDestroy(g);
    return rc;
  }
  if (e) return cuda_fail(e, "cudaStreamEndCapture");
  bpm_exec* x = new bpm_exec();
  x->graph = g;
  x->launches = n;
  e = cudaGraphInstantiate(&x->exec, g, 0);
  if (e) {
    cudaGraphDestroy(g);
    delete x;
    return cuda_fail(e, "cudaGraphInstantiate");
  }
  *out = x;
  return BPM_OK;
}

extern "C" int bpm_exec_launch(bpm_exec* x, void* stream) {
  clear_error();
  if (!x) { set_error("exec is NULL"); return BPM_ERR_ARG; }
  BPM_CUDA_TRY(cudaGraphLaunch(x->exec, static_cast<cudaStream_t>(stream)));
  count_launch(x->launches);
  return BPM_OK;
}

extern "C" int bpm_exec_destroy(bpm_exec* x) {
  if (!x) return BPM_OK;
  cudaGraphExecDestroy(x->exec);
  cudaGraphDestroy(x->graph);
  delete x;
  return BPM_OK;
}

// ---------------------------------------------------------------------------------------
// Allocation-free march.
//
// Some callers cannot allocate device memory at the point where they march: a host
// application that hands this library a fixed device memory budget and forbids it any
// cudaMalloc of its own, a plugin whose host owns every device allocation, or a caller in
// a latency-critical loop where cudaMalloc (which synchronises the device) would stall
// the streams running beside it. For them, bpm_propagate_noalloc takes its scratch from
// one fixed array in this library's device image instead of a caller workspace. Every GPU
// that loads the library holds that array (BPM_NOALLOC_SCRATCH_BYTES) until the process
// exits.
// ---------------------------------------------------------------------------------------
#include <mutex>

static __device__ __align__(256) unsigned char g_noalloc_scratch[BPM_NOALLOC_SCRATCH_BYTES];

namespace {
constexpr int kMaxDevices = 64;
std::mutex g_noalloc_mu;
void* g_noalloc_addr[kMaxDevices] = {};

// Device address of g_noalloc_scratch on the current device. In host code the symbol is
// only a host-side stand-in, so it is never passed to a kernel: its device address is
// looked up once per device, with that device current, and cached.
int noalloc_scratch(void** out) {
  int dev = -1;
  BPM_CUDA_TRY(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDevices) {
    set_error("device index out of range for the allocation-free scratch");
    return BPM_ERR_ARG;
  }
  std::lock_guard<std::mutex> lock(g_noalloc_mu);
  if (!g_noalloc_addr[dev]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(g_noalloc_scratch)");
    g_noalloc_addr[dev] = p;
  }
  *out = g_noalloc_addr[dev];
  return BPM_OK;
}
}  // namespace

extern "C" int bpm_propagate_noalloc(bpm_plan* pl, const bpm_request* r, void* stream) {
  clear_error();
  if (!pl) { set_error("plan is NULL"); return BPM_ERR_ARG; }
  int rc = check_request(pl, r);
  if (rc) return rc;
  // the scratch array is looked up on the current device, and the plan's tables and
  // streams live on the device it was created on: the two must be the same
  {
    int dev = -1;
    BPM_CUDA_TRY(cudaGetDevice(&dev));
    if (dev != pl->device) {
      set_error("bpm_propagate_noalloc: the plan belongs to device " + std::to_string(pl->device) +
                " but device " + std::to_string(dev) + " is current; make the plan's device current");
      return BPM_ERR_ARG;
    }
  }
  // march as many fields together as the fixed scratch holds (the result does not depend
  // on the grouping); refuse grids whose single-field scratch does not fit
  int G = group_size(pl, r);
  while (G > 1 && ws_layout(pl, G).total > BPM_NOALLOC_SCRATCH_BYTES) G--;
  const size_t need = ws_layout(pl, G).total;
  if (need > BPM_NOALLOC_SCRATCH_BYTES) {
    set_error("bpm_propagate_noalloc: a " + std::to_string(pl->d.nx) + "x" + std::to_string(pl->d.ny) +
              " grid needs " + std::to_string(need) + " bytes of scratch, more than its fixed " +
              std::to_string((size_t)BPM_NOALLOC_SCRATCH_BYTES) + " bytes; use bpm_propagate with a workspace");
    return BPM_ERR_OOM;
  }
  void* scratch = nullptr;
  if ((rc = noalloc_scratch(&scratch))) return rc;
  bpm_request q = *r;
  q.group = G;
  return enqueue_march(pl, &q, scratch, BPM_NOALLOC_SCRATCH_BYTES, static_cast<cudaStream_t>(stream));
}
