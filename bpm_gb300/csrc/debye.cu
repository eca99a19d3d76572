// Vectorial Debye-Wolf focus field on GB300 (sm_103a).
//
// Reference: bpm/psf/_focus_fields_debye.py:focus_field_debye (:48-146) launches
// bpm/psf/kernels/psf_debye.cl:debye_wolf (:24-113) over the (Nz0/2+1, Ny0/2+1, Nx0/2+1)
// octant; every work item sums, over INT_STEPS+1 trapezoid nodes t of each annulus,
//   I0 += p(t) (1+cos t) J0(kr sin t) e^{i kz cos t}
//   I1 += p(t) sin t     J1(kr sin t) e^{i kz cos t}
//   I2 += p(t) (cos t-1) J2(kr sin t) e^{i kz cos t},   p(t) = w dt sqrt(cos t)
// and assembles ex, ey, ez, |E|^2; the host then spreads the octant over the full volume.
//
// GB300 design. The sum factorises: I_n(m, z) = sum_t A_n(t, m) E(t, z) with
// A_n(t, m) = p_n(t) J_n(kr_m sin t) over the radii m of the octant's (x, y) columns and
// E(t, z) = e^{i kz_z cos t}. So the quadrature is three real-by-complex matrix products
// sharing E, computed by a register-tiled FP32 FMA kernel; the Bessel functions are
// evaluated once per (node, radius) instead of once per (node, voxel), and the phases
// once per (node, z). Node weights, radii, angles and phases are computed in FP64 (the
// large kz cos t phase is reduced in FP64 before narrowing). A final kernel writes the
// full volume directly, mirroring each voxel to its octant sample (index |m - N0/2|,
// conjugate where z <= Nz0/2, as the reference's slice loop does), so no octant buffer
// and no host-side spreading is needed.
//
// The three products run on the tensor cores (tcgen05.mma, kind::tf32, operands staged by
// TMA, accumulators in tensor memory) in a 3xTF32 split that keeps FP32 accuracy: with
// A = Ah + Al and B = Bh + Bl, Ah and Bh exact TF32 values, D = Ah Bh + Ah Bl + Al Bh (the
// dropped Al Bl is below 2^-20 of the product). Where the octant's x and y grids coincide
// (dx = dy, nx = ny) the integrals depend on the radius only through x^2 + y^2 and the
// rows of A are the distinct (min, max) index pairs of the octant's columns, nxo (nxo + 1)
// / 2 of them instead of nxo^2. BPM_GB300_DEBYE=fma selects the FP32 FMA kernel instead.
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <algorithm>
#include <atomic>
#include <vector>

#include "common.cuh"
#include "tcgen05.cuh"

using namespace bpmgb;

namespace {

constexpr int MAX_NA = 16;

// Pupil weight of each quadrature node.
//   W_STD:   psf_debye.cl:70-75, half weight at i = 0 and i = INT_STEPS, dt sqrt(cos t)
//   W_SINE:  psf_debye.cl:155-159 / :240-244, half weight where the float32 angle equals an
//            annulus limit, dt sqrt(cos t) sin t (debye_wolf_plane, debye_wolf_at)
//   W_GAUSS: psf_debye.cl:336-339, W_SINE times exp(t^2 * gauss_prefac)
//   W_PHYS:  the Debye integral's own pupil factor sqrt(cos t) sin t with an exact
//            trapezoid over [a1, a2]: INT_STEPS nodes t = a1 + i dt, dt = (a2 - a1) /
//            (INT_STEPS - 1), half weight at both ends, the node i = INT_STEPS (past a2)
//            weighted 0 (the formula of tests/test_psf_vectorial.py:15-42 in the reference)
enum WeightKind { W_STD = 0, W_SINE = 1, W_GAUSS = 2, W_PHYS = 3 };

struct NodeArgs {
  float alpha[MAX_NA];
  int n_ann;
  int steps;
  int kind;
  double gauss_prefac;
};

// Octant (or plane) grid: x = x1 + i*(x2-x1)/(N-1.f) per axis
struct OctGeom {
  int nxo, nyo, nzo;
  float x1, x2, y1, y2, z1, z2;
};

// Mirroring of the octant onto the full volume
//   MIR_STD:   focus_field_debye (:116-144), full index m -> |m - N0/2|, conj for z <= Nz0/2
//   MIR_GAUSS: focus_field_debye_gauss (:426-438), p -> p - (N0-N) for p >= N0-N else
//              N-1-p, no conjugation
enum MirrorKind { MIR_STD = 0, MIR_GAUSS = 1 };

struct DebyeLayout {
  size_t si, ct, wf, kr, trig, J, E, I, total;
  int T, M, Zo, nxo, nyo, nzo;
  int Mp, Zp;  // row pitches of J (radii, multiple of 4) and E (planes, even): 16-byte rows
};

DebyeLayout debye_layout(const debye_desc* d, bool gauss = false) {
  DebyeLayout L;
  if (gauss) {
    L.nxo = (d->nx + 1) / 2;
    L.nyo = (d->ny + 1) / 2;
    L.nzo = (d->nz + 1) / 2;
  } else {
    L.nxo = d->nx / 2 + 1;
    L.nyo = d->ny / 2 + 1;
    L.nzo = d->nz / 2 + 1;
  }
  L.T = (d->n_na / 2) * (d->n_integration_steps + 1);
  L.M = L.nxo * L.nyo;
  L.Zo = L.nzo;
  L.Mp = (L.M + 3) & ~3;
  L.Zp = (L.Zo + 1) & ~1;
  size_t off = 0;
  L.si = off; off += align256(sizeof(double) * L.T);
  L.ct = off; off += align256(sizeof(double) * L.T);
  L.wf = off; off += align256(sizeof(float) * 3 * L.T);
  L.kr = off; off += align256(sizeof(double) * L.M);
  L.trig = off; off += align256(sizeof(float) * 4 * L.M);
  L.J = off; off += align256(sizeof(float) * 3 * (size_t)L.T * L.Mp);
  L.E = off; off += align256(sizeof(float2) * (size_t)L.T * L.Zp);
  L.I = off; off += align256(sizeof(float2) * 3 * (size_t)L.Zo * L.M);
  L.total = off;
  return L;
}

// x = x1 + i*(x2-x1)/(N-1.f), FP32 as the kernels evaluate it (psf_debye.cl:46-48)
__device__ __forceinline__ float coord_f32(int i, float x1, float x2, int N) {
  return __fadd_rn(x1, __fdiv_rn(__fmul_rn((float)i, __fsub_rn(x2, x1)), __fsub_rn((float)N, 1.f)));
}

constexpr double kTwoPi = 6.283185307179586, kInvTwoPi = 0.15915494309189535;

// trapezoid node idx of its annulus (psf_debye.cl:62-78), FP64: sin t, cos t and the pupil
// weight w
__device__ __forceinline__ void node_values(const NodeArgs& a, int idx, double& s, double& c, double& w) {
  const int per = a.steps + 1;
  const int ann = idx / per, i = idx - ann * per;
  const double a1 = a.alpha[2 * ann], a2 = a.alpha[2 * ann + 1];
  const double dt = (a2 - a1) / (a.steps - 1.);
  const double t = a1 + i * dt;
  sincos(t, &s, &c);
  if (a.kind == W_STD) {
    w = ((i == 0 || i == a.steps) ? .5 : 1.) * dt * sqrt(c);
  } else if (a.kind == W_PHYS) {
    w = (i == a.steps ? 0. : ((i == 0 || i == a.steps - 1) ? .5 : 1.)) * dt * sqrt(c) * s;
  } else {
    // the end test runs on the float32 angle, each operation rounded on its own
    const float a1f = a.alpha[2 * ann], a2f = a.alpha[2 * ann + 1];
    const float dtf = __fdiv_rn(__fsub_rn(a2f, a1f), __fsub_rn((float)a.steps, 1.f));
    const float tf = __fadd_rn(a1f, __fmul_rn((float)i, dtf));
    w = ((tf == a1f || tf == a2f) ? .5 : 1.) * dt * sqrt(c) * s;
    if (a.kind == W_GAUSS) w *= exp(t * t * a.gauss_prefac);
  }
}

// the per-order node factors p_0 = w (cos t + 1), p_1 = w sin t, p_2 = w (cos t - 1)
__device__ __forceinline__ void node_store(float* wf, int T, int idx, double s, double c, double w) {
  wf[idx] = (float)(w * (c + 1.));
  wf[T + idx] = (float)(w * s);
  wf[2 * T + idx] = (float)(w * (c - 1.));
}

__global__ void debye_nodes_kernel(NodeArgs a, double* si, double* ct, float* wf, int T) {
  int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= T) return;
  double s, c, w;
  node_values(a, idx, s, c, w);
  si[idx] = s;
  ct[idx] = c;
  node_store(wf, T, idx, s, c, w);
}

// k r of octant column m in FP64, and (cos phi, sin phi, cos 2 phi, sin 2 phi) of its azimuth
// from the coordinates: x / r, y / r, (x - y)(x + y) / r^2, 2 x y / r^2 (phi = 0 at the origin,
// as atan2(0, 0))
__device__ __forceinline__ double radius_values(const OctGeom& g, double k, int m, float4& trig) {
  const int jy = m / g.nxo, ix = m - jy * g.nxo;
  const double x = coord_f32(ix, g.x1, g.x2, g.nxo), y = coord_f32(jy, g.y1, g.y2, g.nyo);
  const double r2 = x * x + y * y;
  if (r2 == 0.) {
    trig = make_float4(1.f, 0.f, 1.f, 0.f);
    return 0.;
  }
  const double r = sqrt(r2), ir = 1. / r, ir2 = ir * ir;
  trig = make_float4((float)(x * ir), (float)(y * ir), (float)((x - y) * (x + y) * ir2), (float)(2. * x * y * ir2));
  return k * r;
}

__device__ __forceinline__ void trig_store(float* trig, int M, int m, float4 v) {
  trig[m] = v.x;
  trig[M + m] = v.y;
  trig[2 * M + m] = v.z;
  trig[3 * M + m] = v.w;
}

// radius and azimuth per octant column (ix, jy)
__global__ void debye_radii_kernel(OctGeom g, double k, double* kr, float* trig, int M) {
  int m = blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= M) return;
  float4 tv;
  kr[m] = radius_values(g, k, m, tv);
  trig_store(trig, M, m, tv);
}

// E(t, z) = exp(i kz cos t), phase formed and reduced in FP64
__global__ void debye_phase_kernel(int Zo, int Zp, float z1, float z2, double k, const double* ct, float2* E,
                                   int T) {
  int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= T * Zp) return;
  const int t = idx / Zp, z = idx - t * Zp;
  if (z >= Zo) {  // row padding
    E[idx] = make_float2(0.f, 0.f);
    return;
  }
  const double kz = k * (double)(Zo == 1 ? z1 : coord_f32(z, z1, z2, Zo));
  double s, c;
  sincos(kz * ct[t], &s, &c);
  E[idx] = make_float2((float)c, (float)s);
}

// Coefficients of Hankel's asymptotic expansion (Abramowitz & Stegun 9.2.5, 9.2.9, 9.2.10):
// a_k(n) = prod_{j=1..k} (4 n^2 - (2j - 1)^2) / (8 j), so that for large x
//   J_n(x) = sqrt(2 / (pi x)) (P_n cos chi_n - Q_n sin chi_n), chi_n = x - (n/2 + 1/4) pi,
//   P_n = sum_k (-1)^k a_2k x^-2k,  Q_n = sum_k (-1)^k a_2k+1 x^-(2k+1).
__host__ __device__ constexpr double hankel_a(int n, int k) {
  double a = 1.;
  for (int j = 1; j <= k; j++) a *= (4. * n * n - (2. * j - 1.) * (2. * j - 1.)) / (8. * j);
  return a;
}

// J2 from J0, J1: ascending series for small x, the three-term recurrence J2 = 2 J1/x - J0
// otherwise (stable for n = 2 < x).
__device__ __forceinline__ float bessel_j2(float x, float j0, float j1) {
  const float ax = fabsf(x);
  if (ax < 4.f) {
    // J2(x) = sum_k (-1)^k (x/2)^(2k+2) / (k! (k+2)!)
    const float q = 0.25f * x * x;
    float term = 0.5f * q;  // k = 0: (x/2)^2 / 2!
    float sum = term;
#pragma unroll
    for (int k = 1; k < 12; k++) {
      term *= -q * (1.f / (float)(k * (k + 2)));  // the reciprocal folds to a constant
      sum += term;
    }
    return sum;
  }
  return 2.f * j1 / x - j0;
}

// J0, J1 and J2 together. From x = 16 on, the expansion above truncated after x^-7 (its
// error, below 2e-9 of the envelope sqrt(2 / (pi x)), is under FP32 rounding), with one
// sincosf of x for both orders: chi_0 = x - pi/4 and chi_1 = chi_0 - pi/2, so cos chi_0 =
// (cos x + sin x) / sqrt 2, sin chi_0 = (sin x - cos x) / sqrt 2, cos chi_1 = sin chi_0,
// sin chi_1 = -cos chi_0; 1/x and the envelope come from the approximate reciprocal and
// reciprocal square root (2 ulp, far below what the truncated series resolves), and J2 from
// the recurrence 2 J1/x - J0 with that reciprocal. Below 16: CUDA's j0f and j1f, J2 by
// bessel_j2.
__device__ __forceinline__ void bessel_j012(float x, float& j0, float& j1, float& j2) {
  const float ax = fabsf(x);
  if (ax < 16.f) {
    j0 = j0f(x);
    j1 = j1f(x);
    j2 = bessel_j2(x, j0, j1);
    return;
  }
  const float r = __fdividef(1.f, ax), y = r * r;
  const float P0 = fmaf(fmaf(fmaf((float)-hankel_a(0, 6), y, (float)hankel_a(0, 4)), y, (float)-hankel_a(0, 2)), y, 1.f);
  const float Q0 = r * fmaf(fmaf(fmaf((float)-hankel_a(0, 7), y, (float)hankel_a(0, 5)), y, (float)-hankel_a(0, 3)), y,
                            (float)hankel_a(0, 1));
  const float P1 = fmaf(fmaf(fmaf((float)-hankel_a(1, 6), y, (float)hankel_a(1, 4)), y, (float)-hankel_a(1, 2)), y, 1.f);
  const float Q1 = r * fmaf(fmaf(fmaf((float)-hankel_a(1, 7), y, (float)hankel_a(1, 5)), y, (float)-hankel_a(1, 3)), y,
                            (float)hankel_a(1, 1));
  float s, c;
  sincosf(ax, &s, &c);
  constexpr float kInvSqrt2 = 0.70710678118654752f;
  const float c0 = (c + s) * kInvSqrt2, s0 = (s - c) * kInvSqrt2;   // cos, sin of x - pi/4
  const float env = 0.79788456080286536f * rsqrtf(ax);              // sqrt(2 / (pi x))
  j0 = env * fmaf(P0, c0, -(Q0 * s0));
  const float j1a = env * fmaf(P1, s0, Q1 * c0);                    // P1 cos chi_1 - Q1 sin chi_1
  j1 = x < 0.f ? -j1a : j1a;                                        // J1 is odd
  j2 = fmaf(2.f * r, j1a, -j0);                                     // J2 is even
}

// A_n(t, m) = p_n(t) J_n(kr_m sin t_t)
__global__ void debye_bessel_kernel(int T, int M, int Mp, const double* si, const double* kr, const float* wf,
                                    float* J) {
  const int m = blockIdx.x * blockDim.x + threadIdx.x;
  const int t = blockIdx.y;
  if (m >= Mp) return;
  const size_t TM = (size_t)T * Mp, o = (size_t)t * Mp + m;
  if (m >= M) {  // row padding
    J[o] = J[TM + o] = J[2 * TM + o] = 0.f;
    return;
  }
  const float x = (float)(kr[m] * si[t]);
  float j0, j1;
  float j2;
  bessel_j012(x, j0, j1, j2);
  J[o] = wf[t] * j0;
  J[TM + o] = wf[T + t] * j1;
  J[2 * TM + o] = wf[2 * T + t] * j2;
}

// I_n(z, m) = sum_t A_n(t, m) E(t, z): tile of 64 radii x 32 planes per block, each thread
// owning 4 radii x 2 planes x 3 components. The node slices of A and E are double-buffered
// in shared memory: while the block multiplies slice k, cp.async fetches slice k+1 (rows
// past the last node, radius or plane are zero-filled), so the loads of one slice hide
// behind the arithmetic of the previous one.
constexpr int AM = 64, AZ = 32, AT = 16;
constexpr int ACC_STAGE_F = 3 * AT * AM + 2 * AT * AZ;  // floats per stage: A slice, E slice
constexpr size_t ACC_SMEM = 2 * ACC_STAGE_F * sizeof(float);

__global__ void __launch_bounds__(256, 2) debye_accum_kernel(int T, int M, int Mp, int Zo, int Zp,
                                                             const float* __restrict__ J,
                                                             const float2* __restrict__ E,
                                                             float2* __restrict__ I) {
  extern __shared__ __align__(16) float acc_smem[];
  const int tid = threadIdx.x;
  const int tm = tid & 15, tz = tid >> 4;
  const int m0 = blockIdx.x * AM, z0 = blockIdx.y * AZ;
  const size_t TM = (size_t)T * Mp;
  // one slice of nodes [t0, t0 + AT) into stage st: A rows are 16 pieces of 16 bytes (64
  // radii), E rows 16 pieces (32 planes of complex64)
  auto issue = [&](int st, int t0) {
    float* Js = acc_smem + st * ACC_STAGE_F;
    float* Es = Js + 3 * AT * AM;
    for (int c = tid; c < 3 * AT * 16; c += 256) {
      const int n = c / (AT * 16), r = c - n * AT * 16;
      const int tt = r >> 4, q = r & 15;
      const int t = t0 + tt, m = m0 + q * 4;
      const bool ok = t < T && m < Mp;
      cp_async16_zfill(Js + (n * AT + tt) * AM + q * 4, ok ? J + n * TM + (size_t)t * Mp + m : J, ok ? 16 : 0);
    }
    for (int c = tid; c < AT * 16; c += 256) {
      const int tt = c >> 4, q = c & 15;
      const int t = t0 + tt, z = z0 + q * 2;
      const bool ok = t < T && z < Zp;
      cp_async16_zfill(Es + (tt * AZ + q * 2) * 2, ok ? E + (size_t)t * Zp + z : E, ok ? 16 : 0);
    }
    cp_async_commit();
  };
  float2 acc[3][4][2];
#pragma unroll
  for (int n = 0; n < 3; n++)
#pragma unroll
    for (int a = 0; a < 4; a++)
#pragma unroll
      for (int b = 0; b < 2; b++) acc[n][a][b] = make_float2(0.f, 0.f);
  issue(0, 0);
  for (int k = 0, t0 = 0; t0 < T; k++, t0 += AT) {
    if (t0 + AT < T)
      issue((k + 1) & 1, t0 + AT);
    else
      cp_async_commit();  // keep one group per iteration
    cp_async_wait<1>();   // slice k has landed (slice k+1 may be in flight)
    __syncthreads();
    const float* Js = acc_smem + (k & 1) * ACC_STAGE_F;
    const float2* Es = reinterpret_cast<const float2*>(Js + 3 * AT * AM);
#pragma unroll 4
    for (int tt = 0; tt < AT; tt++) {
      const float4 e4 = *reinterpret_cast<const float4*>(&Es[tt * AZ + tz * 2]);
      const float2 ev[2] = {make_float2(e4.x, e4.y), make_float2(e4.z, e4.w)};
#pragma unroll
      for (int n = 0; n < 3; n++) {
        const float4 j4 = *reinterpret_cast<const float4*>(&Js[(n * AT + tt) * AM + tm * 4]);
        const float jv[4] = {j4.x, j4.y, j4.z, j4.w};
#pragma unroll
        for (int a = 0; a < 4; a++)
#pragma unroll
          for (int b = 0; b < 2; b++) {
            acc[n][a][b].x = fmaf(jv[a], ev[b].x, acc[n][a][b].x);
            acc[n][a][b].y = fmaf(jv[a], ev[b].y, acc[n][a][b].y);
          }
      }
    }
    __syncthreads();  // this stage is refilled two slices later
  }
  cp_async_wait<0>();
  const size_t ZM = (size_t)Zo * M;
#pragma unroll
  for (int n = 0; n < 3; n++)
#pragma unroll
    for (int b = 0; b < 2; b++) {
      const int z = z0 + tz * 2 + b;
      if (z >= Zo) continue;
#pragma unroll
      for (int a = 0; a < 4; a++) {
        const int m = m0 + tm * 4 + a;
        if (m < M) I[n * ZM + (size_t)z * M + m] = acc[n][a][b];
      }
    }
}

// The last nrz (<= RZ) octant planes when they are all that is left after whole 32-plane
// tiles (the host launches it for a single plane). The octant of an even shape has Nz/2 + 1 planes (129 at 256^3): one more 32-plane
// tile for a single plane would cost a full tile's arithmetic, and at 256^3 a fifth wave
// of blocks. Here the product is a matrix-vector one over the nodes, bound by reading A
// with few loads in flight per thread: a block takes 16 radii (4 lanes of 4) and splits
// the nodes over its 64 thread rows (row r takes t = r, r + 64, ...), so each thread's
// chain of dependent loads is T/64 long; the 64 partial sums are then added in row order,
// so the result does not depend on timing.
constexpr int REM_LANES = 4, REM_ROWS = 256 / REM_LANES, REM_M = 4 * REM_LANES;

template <int RZ>
__global__ void __launch_bounds__(256) debye_accum_rem_kernel(int T, int M, int Mp, int Zo, int Zp, int nrz,
                                                              const float* __restrict__ J,
                                                              const float2* __restrict__ E,
                                                              float2* __restrict__ I) {
  __shared__ float2 red[REM_ROWS][REM_M];
  const int tid = threadIdx.x;
  const int tl = tid % REM_LANES, tr = tid / REM_LANES;
  const int m0 = blockIdx.x * REM_M;
  const int ma = m0 + tl * 4;  // first of this lane's 4 radii; Mp is a multiple of 4
  const int zb = Zo - nrz;
  const size_t TM = (size_t)T * Mp;
  float2 acc[3][4][RZ];
#pragma unroll
  for (int n = 0; n < 3; n++)
#pragma unroll
    for (int a = 0; a < 4; a++)
#pragma unroll
      for (int j = 0; j < RZ; j++) acc[n][a][j] = make_float2(0.f, 0.f);
  if (ma < Mp) {
#pragma unroll 4
    for (int t = tr; t < T; t += REM_ROWS) {
      float2 ev[RZ];
#pragma unroll
      for (int j = 0; j < RZ; j++)
        ev[j] = j < nrz ? __ldg(E + (size_t)t * Zp + zb + j) : make_float2(0.f, 0.f);
#pragma unroll
      for (int n = 0; n < 3; n++) {
        const float4 j4 = __ldg(reinterpret_cast<const float4*>(J + n * TM + (size_t)t * Mp + ma));
        const float jv[4] = {j4.x, j4.y, j4.z, j4.w};
#pragma unroll
        for (int a = 0; a < 4; a++)
#pragma unroll
          for (int j = 0; j < RZ; j++) {
            acc[n][a][j].x = fmaf(jv[a], ev[j].x, acc[n][a][j].x);
            acc[n][a][j].y = fmaf(jv[a], ev[j].y, acc[n][a][j].y);
          }
      }
    }
  }
  const size_t ZM = (size_t)Zo * M;
#pragma unroll
  for (int n = 0; n < 3; n++)
#pragma unroll
    for (int j = 0; j < RZ; j++) {
      if (j >= nrz) break;
#pragma unroll
      for (int a = 0; a < 4; a++) red[tr][tl * 4 + a] = acc[n][a][j];
      __syncthreads();
      if (tid < REM_M) {
        float2 s = red[0][tid];
        for (int r = 1; r < REM_ROWS; r++) {
          s.x += red[r][tid].x;
          s.y += red[r][tid].y;
        }
        const int m = m0 + tid;
        if (m < M) I[n * ZM + (size_t)(zb + j) * M + m] = s;
      }
      __syncthreads();
    }
}

// The fields and intensity of octant sample (ix, jy, kz), psf_debye.cl:90-101, unconjugated
struct Voxel {
  float u;
  float2 ex, ey, ez;
};
__device__ __forceinline__ Voxel octant_sample(int ix, int jy, int kz, int nxo, int M, int Zo, float ex0, float ey0,
                                               const float2* __restrict__ I, const float* __restrict__ trig) {
  const int m = jy * nxo + ix;
  const size_t ZM = (size_t)Zo * M, o = (size_t)kz * M + m;
  const float2 I0 = __ldg(I + o), I1 = __ldg(I + ZM + o), I2 = __ldg(I + 2 * ZM + o);
  const float c1 = __ldg(trig + m), s1 = __ldg(trig + M + m);
  const float c2 = __ldg(trig + 2 * M + m), s2 = __ldg(trig + 3 * M + m);
  Voxel r;
  r.ex = make_float2(ex0 * (I0.x + I2.x * c2) + (ey0 * s2) * I2.x, ex0 * (I0.y + I2.y * c2) + (ey0 * s2) * I2.y);
  r.ey = make_float2(ey0 * (I0.x - I2.x * c2) + (ex0 * s2) * I2.x, ey0 * (I0.y - I2.y * c2) + (ex0 * s2) * I2.y);
  const float pz = ex0 * c1 + ey0 * s1;
  r.ez = make_float2(2.f * I1.y * pz, -2.f * I1.x * pz);
  r.u = cabs2(r.ex) + cabs2(r.ey) + cabs2(r.ez);
  return r;
}

// Gather form: the voxel (x, y, z) of the full volume from the octant sample it mirrors onto
// (conjugated fields where MIR_STD asks for it)
template <int MIR>
__device__ __forceinline__ Voxel assemble_point(int x, int y, int z, int nx, int ny, int nz, const OctGeom& g, int M,
                                                int Zo, float ex0, float ey0, const float2* __restrict__ I,
                                                const float* __restrict__ trig) {
  int ix, jy, kz;
  bool conj;
  if (MIR == MIR_STD) {
    ix = abs(x - nx / 2), jy = abs(y - ny / 2), kz = abs(z - nz / 2);
    conj = z <= nz / 2;
  } else {
    ix = x >= nx - g.nxo ? x - (nx - g.nxo) : g.nxo - 1 - x;
    jy = y >= ny - g.nyo ? y - (ny - g.nyo) : g.nyo - 1 - y;
    kz = z >= nz - g.nzo ? z - (nz - g.nzo) : g.nzo - 1 - z;
    conj = false;
  }
  Voxel r = octant_sample(ix, jy, kz, g.nxo, M, Zo, ex0, ey0, I, trig);
  if (conj) {
    r.ex.y = -r.ex.y;
    r.ey.y = -r.ey.y;
    r.ez.y = -r.ez.y;
  }
  return r;
}

// Gather assembly, two neighbouring voxels per thread (even nx) stored as 8- and 16-byte
// vectors: the faster form when the fields are written (470 MB at 256^3), since its paired
// stores beat the scatter form's single ones; each sample is read by every voxel mirroring
// onto it
template <int MIR>
__global__ void debye_assemble_kernel(int nx, int ny, int nz, OctGeom g, int M, int Zo, float ex0, float ey0,
                                      const float2* __restrict__ I, const float* __restrict__ trig,
                                      float* __restrict__ u, float2* __restrict__ ex, float2* __restrict__ ey,
                                      float2* __restrict__ ez) {
  const int y = blockIdx.y, z = blockIdx.z;
  const int x = 2 * (blockIdx.x * blockDim.x + threadIdx.x);
  if (x >= nx) return;
  const Voxel a = assemble_point<MIR>(x, y, z, nx, ny, nz, g, M, Zo, ex0, ey0, I, trig);
  const Voxel b = assemble_point<MIR>(x + 1, y, z, nx, ny, nz, g, M, Zo, ex0, ey0, I, trig);
  const size_t v = ((size_t)z * ny + y) * nx + x;  // even: 8-byte u pairs, 16-byte field pairs
  if (u) __stcs(reinterpret_cast<float2*>(u + v), make_float2(a.u, b.u));
  if (ex) __stcs(reinterpret_cast<float4*>(ex + v), make_float4(a.ex.x, a.ex.y, b.ex.x, b.ex.y));
  if (ey) __stcs(reinterpret_cast<float4*>(ey + v), make_float4(a.ey.x, a.ey.y, b.ey.x, b.ey.y));
  if (ez) __stcs(reinterpret_cast<float4*>(ez + v), make_float4(a.ez.x, a.ez.y, b.ez.x, b.ez.y));
}

// The full-volume positions of octant index q along one axis of N0 points: the inverse of
// the mirroring maps (MIR_STD: q = |p - N0/2|; MIR_GAUSS: q = p - (N0 - N) for p >= N0 - N,
// else N - 1 - q), at most two, in p[0..n)
template <int MIR>
__device__ __forceinline__ int mirror_positions(int q, int N0, int N, int (&p)[2]) {
  int n = 0;
  if (MIR == MIR_STD) {
    const int a = N0 / 2 + q, b = N0 / 2 - q;
    if (a < N0) p[n++] = a;
    if (b >= 0 && b != a) p[n++] = b;
  } else {
    const int a = q + (N0 - N), b = N - 1 - q;
    if (a < N0) p[n++] = a;
    if (b < N0 - N && b >= 0) p[n++] = b;
  }
  return n;
}

// Full-volume assembly fused with the octant mirroring, one octant sample per thread: the
// fields and intensity are formed once (octant_sample) and stored to every
// voxel that mirrors onto the sample (up to 8; conjugated fields where z <= Nz/2 for
// MIR_STD). A warp's 32 consecutive ix store 32 consecutive x on either side of the centre,
// so every store stays coalesced, and the integrals and azimuth tables are read once per
// sample instead of once per voxel (an 8-fold cut of the reads, the whole cost of an
// intensity-only call).
template <int MIR, bool FIELDS>
__global__ void debye_scatter_kernel(int nx, int ny, int nz, OctGeom g, int M, int Zo, float ex0, float ey0,
                                     const float2* __restrict__ I, const float* __restrict__ trig,
                                     float* __restrict__ u, float2* __restrict__ ex, float2* __restrict__ ey,
                                     float2* __restrict__ ez) {
  const int ix = blockIdx.x * blockDim.x + threadIdx.x, jy = blockIdx.y, kz = blockIdx.z;
  if (ix >= g.nxo) return;
  int px[2], py[2], pz[2];
  const int nxp = mirror_positions<MIR>(ix, nx, g.nxo, px);
  const int nyp = mirror_positions<MIR>(jy, ny, g.nyo, py);
  const int nzp = mirror_positions<MIR>(kz, nz, g.nzo, pz);
  if (nxp == 0 || nyp == 0 || nzp == 0) return;
  const Voxel v = octant_sample(ix, jy, kz, g.nxo, M, Zo, ex0, ey0, I, trig);
#pragma unroll
  for (int c = 0; c < 2; c++) {
    if (c >= nzp) break;
    const int z = pz[c];
    const size_t zb = (size_t)z * ny;
    float2 fx = v.ex, fy = v.ey, fz = v.ez;
    if (FIELDS && MIR == MIR_STD && z <= nz / 2) {
      fx.y = -fx.y;
      fy.y = -fy.y;
      fz.y = -fz.y;
    }
#pragma unroll
    for (int b = 0; b < 2; b++) {
      if (b >= nyp) break;
      const size_t row = (zb + py[b]) * nx;
#pragma unroll
      for (int a = 0; a < 2; a++) {
        if (a >= nxp) break;
        const size_t o = row + px[a];
        if (u) __stcs(u + o, v.u);
        if (FIELDS) {
          if (ex) __stcs(ex + o, fx);
          if (ey) __stcs(ey + o, fy);
          if (ez) __stcs(ez + o, fz);
        }
      }
    }
  }
}

// launch the assembly: the paired gather form when fields are written to 16-byte aligned
// buffers of even nx (GB300, 256^3 with all four outputs: gather 82 us against 90 us for the
// scatter form), else one thread per octant sample (intensity only: 0.172 -> 0.151 ms for the
// whole 256^3 PSF)
int launch_assemble(const debye_desc* d, bool gauss, const OctGeom& g, int M, int Zo, const float2* I,
                    const float* trig, float* u, void* ex, void* ey, void* ez, cudaStream_t s) {
  float2 *pex = static_cast<float2*>(ex), *pey = static_cast<float2*>(ey), *pez = static_cast<float2*>(ez);
  const float e0 = (float)d->ex0, e1 = (float)d->ey0;
  const bool fields = ex || ey || ez;
  const bool pair = d->nx % 2 == 0 && ((uintptr_t)u & 7) == 0 && ((uintptr_t)ex & 15) == 0 &&
                    ((uintptr_t)ey & 15) == 0 && ((uintptr_t)ez & 15) == 0;
  if (fields && pair) {
    const dim3 grid((d->nx / 2 + 127) / 128, d->ny, d->nz);
    if (gauss)
      debye_assemble_kernel<MIR_GAUSS><<<grid, 128, 0, s>>>(d->nx, d->ny, d->nz, g, M, Zo, e0, e1, I, trig, u, pex,
                                                            pey, pez);
    else
      debye_assemble_kernel<MIR_STD><<<grid, 128, 0, s>>>(d->nx, d->ny, d->nz, g, M, Zo, e0, e1, I, trig, u, pex,
                                                          pey, pez);
    BPM_LAUNCH_CHECK("debye_assemble_kernel");
    return BPM_OK;
  }
  const dim3 grid((g.nxo + 127) / 128, g.nyo, g.nzo);
  auto fn = gauss ? (fields ? debye_scatter_kernel<MIR_GAUSS, true> : debye_scatter_kernel<MIR_GAUSS, false>)
                  : (fields ? debye_scatter_kernel<MIR_STD, true> : debye_scatter_kernel<MIR_STD, false>);
  fn<<<grid, 128, 0, s>>>(d->nx, d->ny, d->nz, g, M, Zo, e0, e1, I, trig, u, pex, pey, pez);
  BPM_LAUNCH_CHECK("debye_scatter_kernel");
  return BPM_OK;
}

// Fields at arbitrary points (debye_wolf_at, psf_debye.cl:187-269) or on one z plane
// (debye_wolf_plane, :117-183). Without a grid in z the quadrature does not factorise into
// a matrix product, so each thread sums its point's integrand over the nodes, as the
// reference does, with the node tables staged through shared memory. On the plane the
// phase e^{i kz cos t} is one table over the nodes; at free points the argument kz cos t
// is formed and reduced modulo 2 pi in FP64 and the reduced angle goes through sincosf.
struct PointArgs {
  long long n;
  int nx, ny;  // plane grid (GRID only)
  float x1, x2, y1, y2;
  double k;
  float ex0, ey0;
  int T;
};

constexpr int PT_THREADS = 128, PT_CHUNK = 256;

template <bool GRID>
__global__ void __launch_bounds__(PT_THREADS) debye_points_kernel(
    PointArgs a, const float* __restrict__ xs, const float* __restrict__ ys, const float* __restrict__ zs,
    const double* __restrict__ si, const double* __restrict__ ct, const float* __restrict__ wf,
    const float2* __restrict__ Et, float* __restrict__ u, float2* __restrict__ ex, float2* __restrict__ ey,
    float2* __restrict__ ez) {
  __shared__ float s_si[PT_CHUNK];
  __shared__ float s_w[3][PT_CHUNK];
  __shared__ double s_ct[GRID ? 1 : PT_CHUNK];
  __shared__ float2 s_E[GRID ? PT_CHUNK : 1];
  const long long p = (long long)blockIdx.x * PT_THREADS + threadIdx.x;
  const bool active = p < a.n;
  float x = 0.f, y = 0.f, z = 0.f;
  if (active) {
    if (GRID) {
      const int j = (int)(p / a.nx), i = (int)(p - (long long)j * a.nx);
      x = coord_f32(i, a.x1, a.x2, a.nx);
      y = coord_f32(j, a.y1, a.y2, a.ny);
    } else {
      x = xs[p];
      y = ys[p];
      z = zs[p];
    }
  }
  const double xd = x, yd = y;
  const float kr = (float)(a.k * sqrt(xd * xd + yd * yd));
  const double kz = a.k * (double)z;
  float2 I0 = make_float2(0.f, 0.f), I1 = I0, I2 = I0;
  for (int t0 = 0; t0 < a.T; t0 += PT_CHUNK) {
    const int nt = min(PT_CHUNK, a.T - t0);
    __syncthreads();
    for (int e = threadIdx.x; e < nt; e += PT_THREADS) {
      s_si[e] = (float)si[t0 + e];
      s_w[0][e] = wf[t0 + e];
      s_w[1][e] = wf[a.T + t0 + e];
      s_w[2][e] = wf[2 * a.T + t0 + e];
      if (GRID)
        s_E[e] = Et[t0 + e];
      else
        s_ct[e] = ct[t0 + e];
    }
    __syncthreads();
    if (!active) continue;
    for (int tt = 0; tt < nt; tt++) {
      const float xb = kr * s_si[tt];
      float j0, j1;
      float j2;
      bessel_j012(xb, j0, j1, j2);
      float2 e;
      if (GRID) {
        e = s_E[tt];
      } else {
        const double arg = kz * s_ct[tt];
        const double q = rint(arg * kInvTwoPi);
        sincosf((float)fma(-q, kTwoPi, arg), &e.y, &e.x);
      }
      const float a0 = s_w[0][tt] * j0, a1 = s_w[1][tt] * j1, a2 = s_w[2][tt] * j2;
      I0.x = fmaf(a0, e.x, I0.x);
      I0.y = fmaf(a0, e.y, I0.y);
      I1.x = fmaf(a1, e.x, I1.x);
      I1.y = fmaf(a1, e.y, I1.y);
      I2.x = fmaf(a2, e.x, I2.x);
      I2.y = fmaf(a2, e.y, I2.y);
    }
  }
  if (!active) return;
  const double phi = atan2(yd, xd);
  double s1d, c1d, s2d, c2d;
  sincos(phi, &s1d, &c1d);
  sincos(2. * phi, &s2d, &c2d);
  const float c1 = (float)c1d, s1 = (float)s1d, c2 = (float)c2d, s2 = (float)s2d;
  const float ex0 = a.ex0, ey0 = a.ey0;
  // psf_debye.cl:254-263
  const float2 vx = make_float2(ex0 * (I0.x + I2.x * c2) + (ey0 * s2) * I2.x,
                                ex0 * (I0.y + I2.y * c2) + (ey0 * s2) * I2.y);
  if (ex) ex[p] = vx;
  if (u) u[p] = cabs2(vx);  // the reference kernel stores |ex|^2 (psf_debye.cl:267)
  if (ey) ey[p] = make_float2(ey0 * (I0.x - I2.x * c2) + (ex0 * s2) * I2.x, ey0 * (I0.y - I2.y * c2) + (ex0 * s2) * I2.y);
  const float pz = ex0 * c1 + ey0 * s1;
  if (ez) ez[p] = make_float2(2.f * I1.y * pz, -2.f * I1.x * pz);
}


// ---------------------------------------------------------------------------------------
// Tensor-core quadrature. Operands are K-major (node index t contiguous) so TMA tiles of
// 32 nodes x 128 rows land in the 128-byte swizzle layout tcgen05.mma reads:
//   A (3 Mr, T): row n Mr + r = p_n(t) J_n(kr_r sin t), r over the radius rows
//   Bh, Bl (2 Zo, T): row 2z = cos(kz_z cos t), row 2z + 1 = sin(kz_z cos t), split into an
//                     exact TF32 high part and the FP32 remainder
// and the product D = A B^T lands in tensor memory as I[(n, r), (z, re/im)].
// ---------------------------------------------------------------------------------------
__device__ int g_tc_status;  // nonzero once a tensor-core wait gave up (bpm_device_status)

__device__ __forceinline__ float tf32_hi(float v) { return __uint_as_float(__float_as_uint(v) & 0xffffe000u); }

// octant column jy * nxo + ix of radius row r: with a symmetric octant (the x and y grids
// equal) the rows are the distinct pairs ix <= jy in triangular order r = jy (jy + 1) / 2 + ix,
// else r is the column itself
__device__ __forceinline__ int radius_column(int r, int nxo, bool sym) {
  if (!sym) return r;
  int b = (int)((sqrtf(8.f * (float)r + 1.f) - 1.f) * .5f);
  while (b * (b + 1) / 2 > r) b--;
  while ((b + 1) * (b + 2) / 2 <= r) b++;
  const int a = r - b * (b + 1) / 2;
  return b * nxo + a;
}

// An FP64 value v as a float pair (hi, lo): hi = v rounded to FP32, lo = v - hi rounded to FP32,
// so hi + lo is v to about 2^-48 relative.
__device__ __forceinline__ float2 split_pair(double v) {
  const float hi = (float)v;
  return make_float2(hi, (float)(v - (double)hi));
}

// a * b of two float pairs, rounded once to FP32: the exact rounding error of a.hi b.hi (an
// FMA) plus the cross terms, added to the rounded product (a.lo b.lo is below 2^-48). The
// result is the FP32 rounding of the FP64 product except where that product lies within
// about 2^-46 of a rounding boundary; it takes FP32 instructions instead of two of the FP64
// pipe, which runs at 1/64 of the FP32 rate on this GPU.
__device__ __forceinline__ float mul_pair(float2 a, float2 b) {
  const float p = __fmul_rn(a.x, b.x);
  const float e = fmaf(a.x, b.x, -p);
  return __fadd_rn(p, fmaf(a.x, b.y, fmaf(a.y, b.x, e)));
}

// Nodes and radii of the tensor-core path in one launch: blocks [0, nbn) one quadrature node
// per thread (as debye_nodes_kernel: cos t in FP64 for the phases, the three node factors,
// sin t as a float pair), the others one octant column per thread (as debye_radii_kernel,
// k r as a float pair). 32-thread blocks spread the FP64 chains over the SMs.
__global__ void debye_setup_tc_kernel(NodeArgs a, OctGeom g, double k, int T, int M, int nbn, double* ct,
                                      float* wf, float2* si2, float2* kr2, float* trig) {
  if ((int)blockIdx.x < nbn) {
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= T) return;
    double sn, c, w;
    node_values(a, idx, sn, c, w);
    ct[idx] = c;
    si2[idx] = split_pair(sn);
    node_store(wf, T, idx, sn, c, w);
  } else {
    const int m = (blockIdx.x - nbn) * blockDim.x + threadIdx.x;
    if (m >= M) return;
    float4 tv;
    kr2[m] = split_pair(radius_values(g, k, m, tv));
    trig_store(trig, M, m, tv);
  }
}

// The operand tables of the product in one launch of 128-thread blocks: block (row, chunk)
// takes nodes chunk*128 .. +127 of one row,
//   rows [0, Zo): Bh/Bl(2z + {0, 1}, t) = high/low parts of (cos, sin)(kz_z cos t), the phase
//     formed and reduced modulo 2 pi in FP64, its sine and cosine in FP32;
//   rows Zo + r: A(n Mr + r, t) = p_n(t) J_n(kr sin t) for n = 0, 1, 2 (debye_bessel_kernel's
//     values, x = kr sin t rounded to FP32 from the pair product).
__global__ void debye_tables_tc_kernel(int T, int Tp, int Mr, int nxo, int sym, int Zo, float z1, float z2, double k,
                                       const double* __restrict__ ct, const float2* __restrict__ si2,
                                       const float2* __restrict__ kr2, const float* __restrict__ wf,
                                       float* __restrict__ A, float* __restrict__ Bh, float* __restrict__ Bl) {
  const int row = blockIdx.x;
  const int t = blockIdx.y * 128 + threadIdx.x;
  if (t >= T) return;
  if (row < Zo) {
    const int z = row;
    const double kz = k * (double)(Zo == 1 ? z1 : coord_f32(z, z1, z2, Zo));
    const double arg = kz * ct[t];
    const double q = rint(arg * kInvTwoPi);
    float c, sn;
    sincosf((float)fma(-q, kTwoPi, arg), &sn, &c);
    const size_t o = (size_t)(2 * z) * Tp + t;
    Bh[o] = tf32_hi(c);
    Bl[o] = c - tf32_hi(c);
    Bh[o + Tp] = tf32_hi(sn);
    Bl[o + Tp] = sn - tf32_hi(sn);
    return;
  }
  const int r = row - Zo;
  const int m = radius_column(r, nxo, sym != 0);
  const float x = mul_pair(kr2[m], si2[t]);
  float j0, j1, j2;
  bessel_j012(x, j0, j1, j2);
  const size_t o = (size_t)r * Tp + t, RT = (size_t)Mr * Tp;
  A[o] = wf[t] * j0;
  A[RT + o] = wf[T + t] * j1;
  A[2 * RT + o] = wf[2 * T + t] * j2;
}

constexpr int TC_BM = 128, TC_BK = 32, TC_THREADS = 128;
constexpr uint64_t TC_WAIT_NS = 2000000000ull;  // a wait gives up after 2 s

// the dynamic shared-memory limit of debye_accum_tc_kernel, raised once to the opt-in
// maximum (less the kernel's static shared memory) so every tile shape and the wait
// self-test launch under it; tiles are sized to stay below TC_SMEM_MAX
constexpr size_t TC_SMEM_MAX = 227 * 1024 - 256;
cudaError_t tc_prepare();

struct TcArgs {
  int T;           // quadrature nodes (the K extent)
  int rows;        // 3 Mr
  int Mr;          // radius rows
  int Zo;          // octant planes
  int BN;          // product columns per block: a multiple of 16, <= 256
  int stages;      // shared-memory pipeline depth
  uint32_t tmem_cols;
  int nacc;        // accumulators in tensor memory (2 or 3), acc_stride columns apart
  int acc_stride;
  int nxo, M, sym; // octant columns per row, octant columns, radius rows deduplicated
  float2* I;       // (3, Zo, M): row r of the product goes to its octant column(s)
  unsigned long long wait_ns;  // limit of every mbarrier wait
  unsigned extra_tx;           // 0; debye_tc_timeout_selftest announces bytes that never arrive
};

__host__ __device__ constexpr uint32_t tc_a_bytes() { return TC_BM * TC_BK * 4; }
__host__ __device__ constexpr uint32_t tc_b_bytes(int BN) { return (uint32_t)BN * TC_BK * 4; }
__host__ __device__ constexpr uint32_t tc_stage_bytes(int BN) { return 2 * tc_a_bytes() + 2 * tc_b_bytes(BN); }
__host__ __device__ constexpr size_t tc_smem_bytes(int BN, int S) {
  return 1024 + (size_t)S * tc_stage_bytes(BN) + (3 * S + 1) * 8 + 16;
}

// One 128-row x BN-column tile of the product per block of 4 warps, a three-role pipeline
// over S shared-memory stages of one 32-node slice each (A, its TF32 remainder, Bh, Bl):
//   warp 0 lane 0  loads: once the products of slice kt - S have released stage kt % S
//                  (tcgen05.commit on empty[s]), TMA loads of A, Bh, Bl complete on full[s];
//   warps 2 and 3  split: once full[s] has landed, A = Ah + Al, Ah (exact TF32) in place and
//                  Al beside it, then an arrival on split[s] (64 arrivals);
//   warp 1 lane 0  products: once split[s] is complete, the 3xTF32 MMAs of the slice, then
//                  tcgen05.commit on empty[s].
// So loads run up to S slices ahead and a slice's split overlaps the previous slice's
// products. The products go to separate accumulators so that each adds fewer terms (the
// tensor core rounds its FP32 sums with a bias that grows with the number of accumulations):
// Ah Bh of even and of odd node slices to two accumulators and the small cross terms to a
// third (with room for two only, Ah Bh to one and the cross terms to the other); the
// epilogue (all 4 warps, 32 tensor-memory lanes each) adds them in FP32 and stores I. Every
// wait is bounded in time: a role that gives up raises the block's abort flag, the others
// stop at their next wait, the block records g_tc_status, waits (bounded) for its own loads
// and products in flight, frees its tensor memory and returns.
__global__ void __launch_bounds__(TC_THREADS, 1)
debye_accum_tc_kernel(const __grid_constant__ CUtensorMap mapA, const __grid_constant__ CUtensorMap mapBh,
                      const __grid_constant__ CUtensorMap mapBl, TcArgs a) {
  extern __shared__ uint8_t tc_smem_raw[];
  uint8_t* sm = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(tc_smem_raw) + 1023) & ~uintptr_t(1023));
  __shared__ int abort_flag;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int S = a.stages;
  const uint32_t AB = tc_a_bytes(), BB = tc_b_bytes(a.BN), SB = tc_stage_bytes(a.BN);
  uint64_t* full = reinterpret_cast<uint64_t*>(sm + (size_t)S * SB);
  uint64_t* split = full + S;
  uint64_t* empty = split + S;
  uint64_t* done = empty + S;
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(done + 1);
  const int m0 = blockIdx.y * TC_BM, n0 = blockIdx.x * a.BN;
  const int KT = (a.T + TC_BK - 1) / TC_BK;
  constexpr int SPLITTERS = 64;  // warps 2 and 3

  if (tid == 0) {
    for (int i = 0; i < S; i++) {
      tc::mbar_init(&full[i], 1);
      tc::mbar_init(&split[i], SPLITTERS);
      tc::mbar_init(&empty[i], 1);
    }
    tc::mbar_init(done, 1);
    tc::fence_mbar_init();
    tc::tma_prefetch_map(&mapA);
    tc::tma_prefetch_map(&mapBh);
    tc::tma_prefetch_map(&mapBl);
    abort_flag = 0;
  }
  if (warp == 0) {
    tc::tmem_alloc(tmem_slot, a.tmem_cols);
    tc::tmem_relinquish();
  }
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = *tmem_slot;
  volatile int* abortv = &abort_flag;
  int issued = 0;  // slices whose loads were issued (warp 0 lane 0)

  if (warp == 0 && lane == 0) {
    // ---- loads ----
    for (int kt = 0; kt < KT && !*abortv; kt++) {
      const int st = kt % S;
      if (kt >= S && !tc::mbar_wait(&empty[st], (uint32_t)(kt / S - 1) & 1u, a.wait_ns)) {
        *abortv = 1;
        break;
      }
      uint8_t* base = sm + (size_t)st * SB;
      tc::mbar_expect_tx(&full[st], AB + 2 * BB + a.extra_tx);
      tc::tma_load_2d(base, &mapA, &full[st], kt * TC_BK, m0);
      tc::tma_load_2d(base + 2 * AB, &mapBh, &full[st], kt * TC_BK, n0);
      tc::tma_load_2d(base + 2 * AB + BB, &mapBl, &full[st], kt * TC_BK, n0);
      issued = kt + 1;
    }
  } else if (warp >= 2) {
    // ---- TF32 split of A ----
    const int sp = tid - 64;
    for (int kt = 0; kt < KT; kt++) {
      const int st = kt % S;
      if (*abortv) break;
      if (!tc::mbar_wait(&full[st], (uint32_t)(kt / S) & 1u, a.wait_ns)) {
        *abortv = 1;
        break;
      }
      uint8_t* base = sm + (size_t)st * SB;
      float4* pa = reinterpret_cast<float4*>(base);
      float4* pl = reinterpret_cast<float4*>(base + AB);
#pragma unroll 4
      for (int i = sp; i < (int)(AB / 16); i += SPLITTERS) {
        const float4 v = pa[i];
        const float4 h = make_float4(tf32_hi(v.x), tf32_hi(v.y), tf32_hi(v.z), tf32_hi(v.w));
        pl[i] = make_float4(v.x - h.x, v.y - h.y, v.z - h.z, v.w - h.w);
        pa[i] = h;
      }
      tc::fence_proxy_async();  // the split operands are visible to the tensor cores
      tc::mbar_arrive(&split[st]);
    }
  } else if (warp == 1 && lane == 0) {
    // ---- products ----
    const uint32_t idesc = tc::idesc_tf32(TC_BM, a.BN);
    for (int kt = 0; kt < KT; kt++) {
      const int st = kt % S;
      if (*abortv) break;
      if (!tc::mbar_wait(&split[st], (uint32_t)(kt / S) & 1u, a.wait_ns)) {
        *abortv = 1;
        break;
      }
      tc::fence_after_sync();
      const uint32_t sa = tc::smem_u32(sm + (size_t)st * SB), sl = sa + AB, sbh = sa + 2 * AB, sbl = sbh + BB;
      const uint32_t big = a.nacc == 3 ? tmem + (uint32_t)((kt & 1) * a.acc_stride) : tmem;
      const uint32_t cross = tmem + (uint32_t)((a.nacc - 1) * a.acc_stride);
#pragma unroll
      for (int k = 0; k < TC_BK / 8; k++) {  // 8 TF32 (32 bytes) of K per instruction
        const uint64_t dah = tc::desc_sw128_kmajor(sa + 32 * k), dal = tc::desc_sw128_kmajor(sl + 32 * k);
        const uint64_t dbh = tc::desc_sw128_kmajor(sbh + 32 * k), dbl = tc::desc_sw128_kmajor(sbl + 32 * k);
        const bool first_big = a.nacc == 3 ? (kt < 2 && k == 0) : (kt == 0 && k == 0);
        tc::mma_tf32(big, dah, dbh, idesc, first_big ? 0u : 1u);
        tc::mma_tf32(cross, dah, dbl, idesc, (kt > 0 || k > 0) ? 1u : 0u);
        tc::mma_tf32(cross, dal, dbh, idesc, 1u);
      }
      tc::mma_commit(&empty[st]);
    }
    tc::mma_commit(done);  // arrives once every product issued has completed
  }
  // every role has left its loop
  __syncthreads();
  bool ok = !*abortv;
  const bool fin = tc::mbar_wait(done, 0, a.wait_ns);
  ok = __syncthreads_and(ok && fin);
  tc::fence_after_sync();
  if (ok) {
    const int row = m0 + warp * 32 + lane;
    const bool rv = row < a.rows;
    const int n = rv ? row / a.Mr : 0, r = rv ? row - n * a.Mr : 0;
    // octant column (ix, jy) of the row and, for a deduplicated row off the diagonal, its
    // mirror (jy, ix): both receive the integrals, so I keeps the plain column layout
    const int m1 = radius_column(r, a.nxo, a.sym != 0);
    const int ix = m1 % a.nxo, jy = m1 / a.nxo;
    const int m2 = (a.sym && ix != jy) ? ix * a.nxo + jy : -1;
    const size_t ob = ((size_t)n * a.Zo) * a.M;
    const uint32_t lane_base = tmem + ((uint32_t)(warp * 32) << 16);
    const bool two_big = a.nacc == 3 && KT > 1;  // the odd-slice accumulator was written
    for (int c0 = 0; c0 < a.BN; c0 += 16) {
      float v[16], w[16], x[16];
      tc::tmem_ld_32x32b_x16(lane_base + (uint32_t)c0, v);
      tc::tmem_ld_32x32b_x16(lane_base + (uint32_t)((a.nacc - 1) * a.acc_stride + c0), x);
      if (two_big) {
        tc::tmem_ld_32x32b_x16(lane_base + (uint32_t)(a.acc_stride + c0), w);
#pragma unroll
        for (int j = 0; j < 16; j++) v[j] += w[j];
      }
#pragma unroll
      for (int j = 0; j < 16; j++) v[j] += x[j];
      if (rv) {
#pragma unroll
        for (int j = 0; j < 8; j++) {
          const int z = (n0 + c0) / 2 + j;
          if (z < a.Zo) {
            const float2 val = make_float2(v[2 * j], v[2 * j + 1]);
            a.I[ob + (size_t)z * a.M + m1] = val;
            if (m2 >= 0) a.I[ob + (size_t)z * a.M + m2] = val;
          }
        }
      }
    }
  } else if (tid == 0) {
    atomicExch(&g_tc_status, 1);
    // loads issued but never consumed still land in this block's shared memory: wait for
    // each stage's latest issued load (bounded) before the block exits
    for (int kt = issued > S ? issued - S : 0; kt < issued; kt++)
      tc::mbar_wait(&full[kt % S], (uint32_t)(kt / S) & 1u, a.wait_ns);
  }
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(tmem, a.tmem_cols);
}

// once per device (the attribute belongs to the current device's context); the opt-in
// limit covers static and dynamic shared memory together
cudaError_t tc_prepare() {
  constexpr int kDevices = 64;
  static std::atomic<bool> done[kDevices];
  int dev = 0, optin = 0;
  cudaError_t r;
  if ((r = cudaGetDevice(&dev))) return r;
  if (dev >= 0 && dev < kDevices && done[dev].load(std::memory_order_acquire)) return cudaSuccess;
  cudaFuncAttributes fa;
  if ((r = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev)) ||
      (r = cudaFuncGetAttributes(&fa, debye_accum_tc_kernel)))
    return r;
  const size_t room = (size_t)optin - fa.sharedSizeBytes;
  r = cudaFuncSetAttribute(debye_accum_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)std::min(room, TC_SMEM_MAX));
  if (r == cudaSuccess && dev >= 0 && dev < kDevices) done[dev].store(true, std::memory_order_release);
  return r;
}

enum Variant { V_STD = 0, V_GAUSS = 1, V_PLANE = 2, V_AT = 3 };

int check_desc(const debye_desc* d, Variant v = V_STD) {
  if (!d) { set_error("description is NULL"); return BPM_ERR_ARG; }
  if (v == V_STD) {
    if (d->nx < 2 || d->ny < 2 || d->nz < 2) { set_error("shape must be >= 2 in every axis"); return BPM_ERR_SHAPE; }
    if (d->nx % 2 + d->ny % 2 + d->nz % 2 != 0) {
      set_error("odd shapes not supported yet");  // _focus_fields_debye.py:81-82
      return BPM_ERR_SHAPE;
    }
  } else if (v == V_GAUSS) {
    // octant (N0+1)/2 >= 2 per axis: the grid divides by (N-1)
    if (d->nx < 3 || d->ny < 3 || d->nz < 3) { set_error("shape must be >= 3 in every axis"); return BPM_ERR_SHAPE; }
  } else if (v == V_PLANE) {
    if (d->nx < 2 || d->ny < 2) { set_error("plane shape must be >= 2 in both axes"); return BPM_ERR_SHAPE; }
  }
  if (d->ny > 65535 || d->nz > 65535) { set_error("ny and nz must be <= 65535"); return BPM_ERR_SHAPE; }
  if (!d->na || d->n_na < 2 || d->n_na % 2 || d->n_na > MAX_NA) {
    set_error("NA must be a scalar or an even-length list of at most 16 values");
    return BPM_ERR_ARG;
  }
  if (d->n_integration_steps < 2) { set_error("n_integration_steps must be >= 2"); return BPM_ERR_ARG; }
  if (d->quadrature != DEBYE_QUAD_REFERENCE && (v != V_STD || d->quadrature != DEBYE_QUAD_PHYSICAL)) {
    set_error("quadrature must be DEBYE_QUAD_REFERENCE, or DEBYE_QUAD_PHYSICAL for debye_focus_field");
    return BPM_ERR_ARG;
  }
  if ((long long)(d->n_na / 2) * (d->n_integration_steps + 1) > 65535) {
    set_error("too many quadrature nodes: (len(NA)/2) * (n_integration_steps+1) must be <= 65535");
    return BPM_ERR_ARG;
  }
  if (!(d->lam > 0) || !(d->n0 > 0)) { set_error("lam and n0 must be positive"); return BPM_ERR_ARG; }
  if ((v == V_STD || v == V_GAUSS || v == V_PLANE) && (!(d->dx > 0) || !(d->dy > 0))) {
    set_error("dx and dy must be positive");
    return BPM_ERR_ARG;
  }
  if ((v == V_STD || v == V_GAUSS) && !(d->dz >= 0)) { set_error("dz must be >= 0"); return BPM_ERR_ARG; }
  return BPM_OK;
}

NodeArgs node_args(const debye_desc* d, int kind) {
  NodeArgs na;
  memset(&na, 0, sizeof(na));
  na.n_ann = d->n_na / 2;
  na.steps = d->n_integration_steps;
  na.kind = kind;
  // alphas = arcsin(NA/n0) cast to float32 (_focus_fields_debye.py:76, :108)
  for (int i = 0; i < d->n_na; i++) na.alpha[i] = (float)asin(d->na[i] / d->n0);
  return na;
}

// lam/n0 as the float32 kernel argument, and 2 pi / lam from it
double wave_number(const debye_desc* d) {
  const float lamf = (float)(1. * d->lam / d->n0);
  return 2. * M_PI / (double)lamf;
}

// the octant pipeline shared by focus_field_debye and focus_field_debye_gauss
// ---- tensor-core path (host) -------------------------------------------------------------
}  // namespace

int bpmgb::tc::encode_f32_kmajor(CUtensorMap* map, const float* base, uint64_t rows, uint64_t cols,
                                 uint64_t pitch_elems, uint32_t box_rows) {
  using EncodeFn = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
  static EncodeFn fn = [] {
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
      f = nullptr;
    cudaGetLastError();
    return reinterpret_cast<EncodeFn>(f);
  }();
  if (!fn) return -1;
  const cuuint64_t dims[2] = {cols, rows};
  const cuuint64_t strides[1] = {pitch_elems * sizeof(float)};
  const cuuint32_t box[2] = {32, box_rows};
  const cuuint32_t estr[2] = {1, 1};
  return (int)fn(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<float*>(base), dims, strides, box, estr,
                 CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                 CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
}

namespace {

// the octant quadrature on the tensor cores unless BPM_GB300_DEBYE=fma
bool debye_tc_enabled() {
  static const bool on = [] {
    const char* e = getenv("BPM_GB300_DEBYE");
    return !(e && strcmp(e, "fma") == 0);
  }();
  return on;
}

// octant grid and node weights shared by both quadrature kernels
void octant_setup(const debye_desc* d, bool gauss, double sig, int nxo, int nyo, int nzo, OctGeom& g, NodeArgs& na) {
  na = node_args(d, gauss ? W_GAUSS : (d->quadrature == DEBYE_QUAD_PHYSICAL ? W_PHYS : W_STD));
  g.nxo = nxo;
  g.nyo = nyo;
  g.nzo = nzo;
  g.x1 = g.y1 = g.z1 = 0.f;
  if (gauss) {
    // _focus_fields_debye.py:404-412: x2 = dx*Nx with Nx the octant size
    g.x2 = (float)(d->dx * nxo);
    g.y2 = (float)(d->dy * nyo);
    g.z2 = (float)(d->dz * nzo);
    // psf_debye.cl:310-311: exp_prefac = -.5/alpha_max^2/sig^2, from the float32 arguments
    const double amax = na.alpha[d->n_na - 1], sg = (float)sig;
    na.gauss_prefac = -.5 / amax / amax / sg / sg;
  } else {
    // _focus_fields_debye.py:102-109
    g.x2 = (float)(d->dx * (nxo - 1.));
    g.y2 = (float)(d->dy * (nyo - 1.));
    g.z2 = (float)(d->dz * (nzo - 1.));
  }
}

struct TcLayout {
  size_t si2, ct, wf, kr2, trig, A, Bh, Bl, I, total;
  int T, Tp, M, Mr, Zo, nxo, nyo, nzo, BN, ntn, stages;
  bool sym;
};

TcLayout tc_layout(const debye_desc* d, bool gauss) {
  TcLayout L;
  if (gauss) {
    L.nxo = (d->nx + 1) / 2;
    L.nyo = (d->ny + 1) / 2;
    L.nzo = (d->nz + 1) / 2;
  } else {
    L.nxo = d->nx / 2 + 1;
    L.nyo = d->ny / 2 + 1;
    L.nzo = d->nz / 2 + 1;
  }
  OctGeom g;
  NodeArgs na;
  octant_setup(d, gauss, 1., L.nxo, L.nyo, L.nzo, g, na);
  L.sym = L.nxo == L.nyo && g.x1 == g.y1 && g.x2 == g.y2;
  L.T = (d->n_na / 2) * (d->n_integration_steps + 1);
  L.Tp = (L.T + 3) & ~3;  // 16-byte rows for TMA
  L.M = L.nxo * L.nyo;
  L.Mr = L.sym ? L.nxo * (L.nxo + 1) / 2 : L.M;
  L.Zo = L.nzo;
  // product columns 2 Zo in ntn blocks of BN (a multiple of 16, <= 256)
  const int cols = 2 * L.Zo;
  L.ntn = (cols + 255) / 256;
  L.BN = ((cols + L.ntn - 1) / L.ntn + 15) & ~15;
  L.stages = tc_smem_bytes(L.BN, 3) <= TC_SMEM_MAX ? 3 : 2;
  size_t off = 0;
  L.si2 = off; off += align256(sizeof(float2) * L.T);
  L.ct = off; off += align256(sizeof(double) * L.T);
  L.wf = off; off += align256(sizeof(float) * 3 * L.T);
  L.kr2 = off; off += align256(sizeof(float2) * L.M);
  L.trig = off; off += align256(sizeof(float) * 4 * L.M);
  L.A = off; off += align256(sizeof(float) * 3 * (size_t)L.Mr * L.Tp);
  L.Bh = off; off += align256(sizeof(float) * 2 * (size_t)L.Zo * L.Tp);
  L.Bl = off; off += align256(sizeof(float) * 2 * (size_t)L.Zo * L.Tp);
  L.I = off; off += align256(sizeof(float2) * 3 * (size_t)L.Zo * L.M);
  L.total = off;
  return L;
}

size_t octant_workspace_bytes(const debye_desc* d, bool gauss) {
  return debye_tc_enabled() ? tc_layout(d, gauss).total : debye_layout(d, gauss).total;
}

int run_octant_tc(const debye_desc* d, bool gauss, double sig, float* u, void* ex, void* ey, void* ez, void* ws,
                  size_t ws_bytes, cudaStream_t s) {
  TcLayout L = tc_layout(d, gauss);
  if (!ws || ws_bytes < L.total) {
    set_error("workspace too small: need " + std::to_string(L.total) + " bytes");
    return BPM_ERR_OOM;
  }
  if (!aligned16(ws)) { set_error("workspace must be 16-byte aligned"); return BPM_ERR_ARG; }
  char* w = static_cast<char*>(ws);
  float2* si2 = reinterpret_cast<float2*>(w + L.si2);
  double* ct = reinterpret_cast<double*>(w + L.ct);
  float* wf = reinterpret_cast<float*>(w + L.wf);
  float2* kr2 = reinterpret_cast<float2*>(w + L.kr2);
  float* trig = reinterpret_cast<float*>(w + L.trig);
  float* A = reinterpret_cast<float*>(w + L.A);
  float* Bh = reinterpret_cast<float*>(w + L.Bh);
  float* Bl = reinterpret_cast<float*>(w + L.Bl);
  float2* I = reinterpret_cast<float2*>(w + L.I);
  OctGeom g;
  NodeArgs na;
  octant_setup(d, gauss, sig, L.nxo, L.nyo, L.nzo, g, na);
  const double k = wave_number(d);
  const int rows = 3 * L.Mr;

  CUtensorMap mA, mBh, mBl;
  if (tc::encode_f32_kmajor(&mA, A, (uint64_t)rows, (uint64_t)L.T, (uint64_t)L.Tp, TC_BM) ||
      tc::encode_f32_kmajor(&mBh, Bh, (uint64_t)2 * L.Zo, (uint64_t)L.T, (uint64_t)L.Tp, (uint32_t)L.BN) ||
      tc::encode_f32_kmajor(&mBl, Bl, (uint64_t)2 * L.Zo, (uint64_t)L.T, (uint64_t)L.Tp, (uint32_t)L.BN)) {
    set_error("cuTensorMapEncodeTiled failed for the quadrature operands");
    return BPM_ERR_CUDA;
  }
  const int tb = (L.T + 127) / 128;
  const int nbn = (L.T + 31) / 32;
  debye_setup_tc_kernel<<<(unsigned)(nbn + (L.M + 31) / 32), 32, 0, s>>>(na, g, k, L.T, L.M, nbn, ct, wf, si2, kr2,
                                                                          trig);
  BPM_LAUNCH_CHECK("debye_setup_tc_kernel");
  debye_tables_tc_kernel<<<dim3((unsigned)(L.Zo + L.Mr), (unsigned)tb), 128, 0, s>>>(
      L.T, L.Tp, L.Mr, L.nxo, L.sym ? 1 : 0, L.Zo, g.z1, g.z2, k, ct, si2, kr2, wf, A, Bh, Bl);
  BPM_LAUNCH_CHECK("debye_tables_tc_kernel");
  TcArgs ta;
  ta.T = L.T;
  ta.rows = rows;
  ta.Mr = L.Mr;
  ta.Zo = L.Zo;
  ta.BN = L.BN;
  ta.stages = L.stages;
  // accumulators 32-column aligned; three when they fit the 512 columns, else two
  ta.acc_stride = (L.BN + 31) & ~31;
  ta.nacc = 3 * ta.acc_stride <= 512 ? 3 : 2;
  {
    uint32_t need = (uint32_t)(ta.nacc * ta.acc_stride), c = 32;
    while (c < need) c <<= 1;
    ta.tmem_cols = c;
  }
  ta.nxo = L.nxo;
  ta.M = L.M;
  ta.sym = L.sym ? 1 : 0;
  ta.I = I;
  ta.wait_ns = TC_WAIT_NS;
  ta.extra_tx = 0;
  const size_t smem = tc_smem_bytes(L.BN, L.stages);
  if (smem > TC_SMEM_MAX) { set_error("quadrature tile does not fit shared memory"); return BPM_ERR_SHAPE; }
  BPM_CUDA_TRY(tc_prepare());
  const dim3 grid(L.ntn, (rows + TC_BM - 1) / TC_BM);
  debye_accum_tc_kernel<<<grid, TC_THREADS, smem, s>>>(mA, mBh, mBl, ta);
  BPM_LAUNCH_CHECK("debye_accum_tc_kernel");
  if (u || ex || ey || ez) return launch_assemble(d, gauss, g, L.M, L.Zo, I, trig, u, ex, ey, ez, s);
  return BPM_OK;
}

int run_octant(const debye_desc* d, bool gauss, double sig, float* u, void* ex, void* ey, void* ez, void* ws,
               size_t ws_bytes, cudaStream_t s) {
  if (debye_tc_enabled()) return run_octant_tc(d, gauss, sig, u, ex, ey, ez, ws, ws_bytes, s);
  DebyeLayout L = debye_layout(d, gauss);
  if (!ws || ws_bytes < L.total) {
    set_error("workspace too small: need " + std::to_string(L.total) + " bytes");
    return BPM_ERR_OOM;
  }
  char* w = static_cast<char*>(ws);
  double* si = reinterpret_cast<double*>(w + L.si);
  double* ct = reinterpret_cast<double*>(w + L.ct);
  float* wf = reinterpret_cast<float*>(w + L.wf);
  double* kr = reinterpret_cast<double*>(w + L.kr);
  float* trig = reinterpret_cast<float*>(w + L.trig);
  float* J = reinterpret_cast<float*>(w + L.J);
  float2* E = reinterpret_cast<float2*>(w + L.E);
  float2* I = reinterpret_cast<float2*>(w + L.I);

  OctGeom g;
  NodeArgs na;
  octant_setup(d, gauss, sig, L.nxo, L.nyo, L.nzo, g, na);
  const double k = wave_number(d);

  debye_nodes_kernel<<<(L.T + 127) / 128, 128, 0, s>>>(na, si, ct, wf, L.T);
  BPM_LAUNCH_CHECK("debye_nodes_kernel");
  debye_radii_kernel<<<(L.M + 127) / 128, 128, 0, s>>>(g, k, kr, trig, L.M);
  BPM_LAUNCH_CHECK("debye_radii_kernel");
  debye_phase_kernel<<<(L.T * L.Zp + 127) / 128, 128, 0, s>>>(L.Zo, L.Zp, g.z1, g.z2, k, ct, E, L.T);
  BPM_LAUNCH_CHECK("debye_phase_kernel");
  debye_bessel_kernel<<<dim3((L.Mp + 127) / 128, L.T), 128, 0, s>>>(L.T, L.M, L.Mp, si, kr, wf, J);
  BPM_LAUNCH_CHECK("debye_bessel_kernel");
  static PerDevice attr;
  attr.get([] {
    cudaFuncSetAttribute(debye_accum_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)ACC_SMEM);
    return 1;
  });
  // whole 32-plane tiles in the tile kernel; a single plane past them (the octant's
  // Nz/2 + 1 planes of a power-of-two shape) in the matrix-vector kernel; other
  // remainders stay a partial tile of the tile kernel
  const int nrz = (L.Zo > AZ && L.Zo % AZ == 1) ? 1 : 0;
  const int mtiles = (L.M + AM - 1) / AM;
  debye_accum_kernel<<<dim3(mtiles, (L.Zo - nrz + AZ - 1) / AZ), 256, ACC_SMEM, s>>>(L.T, L.M, L.Mp, L.Zo, L.Zp, J,
                                                                                   E, I);
  BPM_LAUNCH_CHECK("debye_accum_kernel");
  const int rtiles = (L.M + REM_M - 1) / REM_M;
  if (nrz == 1) {
    debye_accum_rem_kernel<1><<<rtiles, 256, 0, s>>>(L.T, L.M, L.Mp, L.Zo, L.Zp, nrz, J, E, I);
    BPM_LAUNCH_CHECK("debye_accum_rem_kernel");
  }
  if (u || ex || ey || ez) return launch_assemble(d, gauss, g, L.M, L.Zo, I, trig, u, ex, ey, ez, s);
  return BPM_OK;
}

struct PointsLayout {
  size_t si, ct, wf, E, total;
  int T;
};

PointsLayout points_layout(const debye_desc* d) {
  PointsLayout L;
  L.T = (d->n_na / 2) * (d->n_integration_steps + 1);
  size_t off = 0;
  L.si = off; off += align256(sizeof(double) * L.T);
  L.ct = off; off += align256(sizeof(double) * L.T);
  L.wf = off; off += align256(sizeof(float) * 3 * L.T);
  L.E = off; off += align256(sizeof(float2) * L.T);
  L.total = off;
  return L;
}

// shared by focus_field_debye_plane (GRID) and focus_field_debye_at
int run_points(const debye_desc* d, bool grid, double zplane, const float* xs, const float* ys, const float* zs,
               long long n, float* u, void* ex, void* ey, void* ez, void* ws, size_t ws_bytes, cudaStream_t s) {
  PointsLayout L = points_layout(d);
  if (!ws || ws_bytes < L.total) {
    set_error("workspace too small: need " + std::to_string(L.total) + " bytes");
    return BPM_ERR_OOM;
  }
  char* w = static_cast<char*>(ws);
  double* si = reinterpret_cast<double*>(w + L.si);
  double* ct = reinterpret_cast<double*>(w + L.ct);
  float* wf = reinterpret_cast<float*>(w + L.wf);
  float2* E = reinterpret_cast<float2*>(w + L.E);
  NodeArgs na = node_args(d, W_SINE);
  const double k = wave_number(d);
  debye_nodes_kernel<<<(L.T + 127) / 128, 128, 0, s>>>(na, si, ct, wf, L.T);
  BPM_LAUNCH_CHECK("debye_nodes_kernel");
  PointArgs a;
  memset(&a, 0, sizeof(a));
  a.n = n;
  a.k = k;
  a.ex0 = (float)d->ex0;
  a.ey0 = (float)d->ey0;
  a.T = L.T;
  if (n == 0) return BPM_OK;
  const long long blocks = (n + PT_THREADS - 1) / PT_THREADS;
  if (blocks > 0x7fffffffLL) { set_error("too many points"); return BPM_ERR_SHAPE; }
  if (grid) {
    // _focus_fields_debye.py:201-209: x in [-(Nx//2) dx, (Nx - Nx//2) dx], float32
    a.nx = d->nx;
    a.ny = d->ny;
    a.x1 = (float)(-(double)(d->nx / 2) * d->dx);
    a.x2 = (float)((double)(d->nx - d->nx / 2) * d->dx);
    a.y1 = (float)(-(double)(d->ny / 2) * d->dy);
    a.y2 = (float)((double)(d->ny - d->ny / 2) * d->dy);
    debye_phase_kernel<<<(L.T + 127) / 128, 128, 0, s>>>(1, 1, (float)zplane, 0.f, k, ct, E, L.T);
    BPM_LAUNCH_CHECK("debye_phase_kernel");
    debye_points_kernel<true><<<(unsigned)blocks, PT_THREADS, 0, s>>>(a, nullptr, nullptr, nullptr, si, ct, wf, E,
                                                                      u, static_cast<float2*>(ex),
                                                                      static_cast<float2*>(ey),
                                                                      static_cast<float2*>(ez));
  } else {
    debye_points_kernel<false><<<(unsigned)blocks, PT_THREADS, 0, s>>>(a, xs, ys, zs, si, ct, wf, E, u,
                                                                       static_cast<float2*>(ex),
                                                                       static_cast<float2*>(ey),
                                                                       static_cast<float2*>(ez));
  }
  BPM_LAUNCH_CHECK("debye_points_kernel");
  return BPM_OK;
}

}  // namespace

extern "C" size_t debye_workspace_bytes(const debye_desc* d) {
  if (check_desc(d)) return 0;
  return octant_workspace_bytes(d, false);
}

extern "C" int debye_focus_field(const debye_desc* d, float* u, void* ex, void* ey, void* ez, void* ws,
                                 size_t ws_bytes, void* stream) {
  clear_error();
  int rc = check_desc(d);
  if (rc) return rc;
  return run_octant(d, false, 0., u, ex, ey, ez, ws, ws_bytes, static_cast<cudaStream_t>(stream));
}

extern "C" size_t debye_gauss_workspace_bytes(const debye_desc* d) {
  if (check_desc(d, V_GAUSS)) return 0;
  return octant_workspace_bytes(d, true);
}

extern "C" int debye_focus_field_gauss(const debye_desc* d, double sig, float* u, void* ex, void* ey, void* ez,
                                       void* ws, size_t ws_bytes, void* stream) {
  clear_error();
  int rc = check_desc(d, V_GAUSS);
  if (rc) return rc;
  if (!(sig > 0)) { set_error("sig must be > 0"); return BPM_ERR_ARG; }  // _focus_fields_debye.py:387
  return run_octant(d, true, sig, u, ex, ey, ez, ws, ws_bytes, static_cast<cudaStream_t>(stream));
}

extern "C" size_t debye_points_workspace_bytes(const debye_desc* d) {
  if (check_desc(d, V_AT)) return 0;
  return points_layout(d).total;
}

extern "C" int debye_focus_field_plane(const debye_desc* d, double z, void* ex, void* ws, size_t ws_bytes,
                                       void* stream) {
  clear_error();
  int rc = check_desc(d, V_PLANE);
  if (rc) return rc;
  if (!ex) { set_error("ex is NULL"); return BPM_ERR_ARG; }
  return run_points(d, true, z, nullptr, nullptr, nullptr, (long long)d->nx * d->ny, nullptr, ex, nullptr,
                    nullptr, ws, ws_bytes, static_cast<cudaStream_t>(stream));
}

extern "C" int debye_focus_field_at(const debye_desc* d, const float* x, const float* y, const float* z,
                                    long long n, float* u, void* ex, void* ey, void* ez, void* ws,
                                    size_t ws_bytes, void* stream) {
  clear_error();
  int rc = check_desc(d, V_AT);
  if (rc) return rc;
  if (n < 0) { set_error("n must be >= 0"); return BPM_ERR_ARG; }
  if (n > 0 && (!x || !y || !z)) { set_error("coordinate arrays are NULL"); return BPM_ERR_ARG; }
  return run_points(d, false, 0., x, y, z, n, u, ex, ey, ez, ws, ws_bytes, static_cast<cudaStream_t>(stream));
}

extern "C" int bpm_device_status(int clear) {
  int v = 0;
  BPM_CUDA_TRY(cudaMemcpyFromSymbol(&v, g_tc_status, sizeof(int)));
  if (clear && v) {
    const int zero = 0;
    BPM_CUDA_TRY(cudaMemcpyToSymbol(g_tc_status, &zero, sizeof(int)));
  }
  return v;
}

// Self-test of the bounded waits of debye_accum_tc_kernel: one block on a small product whose
// loads announce 16 bytes more than they deliver, so the slice never completes; every wait
// gives up after wait_ms, the block records g_tc_status and leaves with its tensor memory
// freed. Returns BPM_ERR_TIMEOUT when that happened (and clears the status), BPM_OK if the
// product completed, a negative status on a CUDA error. Allocates and frees its own small
// buffers; synchronises the device.
extern "C" int debye_tc_timeout_selftest(double wait_ms) {
  clear_error();
  if (!(wait_ms > 0) || wait_ms > 1000.) { set_error("wait_ms must be in (0, 1000]"); return BPM_ERR_ARG; }
  const int T = 64, Tp = 64, rows = 128, cols = 16;
  float *A = nullptr, *Bh = nullptr, *Bl = nullptr;
  float2* I = nullptr;
  auto release = [&]() {
    cudaFree(A);
    cudaFree(Bh);
    cudaFree(Bl);
    cudaFree(I);
  };
  cudaError_t e;
  if ((e = cudaMalloc(&A, sizeof(float) * rows * Tp)) || (e = cudaMalloc(&Bh, sizeof(float) * cols * Tp)) ||
      (e = cudaMalloc(&Bl, sizeof(float) * cols * Tp)) || (e = cudaMalloc(&I, sizeof(float2) * rows * cols))) {
    release();
    return cuda_fail(e, "cudaMalloc");
  }
  cudaMemset(A, 0, sizeof(float) * rows * Tp);
  cudaMemset(Bh, 0, sizeof(float) * cols * Tp);
  cudaMemset(Bl, 0, sizeof(float) * cols * Tp);
  CUtensorMap mA, mBh, mBl;
  if (tc::encode_f32_kmajor(&mA, A, rows, T, Tp, TC_BM) || tc::encode_f32_kmajor(&mBh, Bh, cols, T, Tp, cols) ||
      tc::encode_f32_kmajor(&mBl, Bl, cols, T, Tp, cols)) {
    release();
    set_error("cuTensorMapEncodeTiled failed");
    return BPM_ERR_CUDA;
  }
  TcArgs ta;
  memset(&ta, 0, sizeof(ta));
  ta.T = T;
  ta.rows = rows;
  ta.Mr = rows / 3 + 1;
  ta.Zo = cols / 2;
  ta.BN = cols;
  ta.stages = 2;
  ta.acc_stride = 32;
  ta.nacc = 3;
  ta.tmem_cols = 128;
  ta.nxo = rows;
  ta.M = rows;
  ta.sym = 0;
  ta.I = I;
  ta.wait_ns = (unsigned long long)(wait_ms * 1e6);
  ta.extra_tx = 16;
  const size_t smem = tc_smem_bytes(ta.BN, ta.stages);
  if ((e = tc_prepare())) {
    release();
    return cuda_fail(e, "cudaFuncSetAttribute");
  }
  debye_accum_tc_kernel<<<dim3(1, 1), TC_THREADS, smem>>>(mA, mBh, mBl, ta);
  if ((e = cudaGetLastError()) || (e = cudaDeviceSynchronize())) {
    release();
    return cuda_fail(e, "debye_accum_tc_kernel (wait self-test)");
  }
  count_launch();
  release();
  int st = bpm_device_status(1);
  if (st < 0) return st;
  return st ? BPM_ERR_TIMEOUT : BPM_OK;
}
