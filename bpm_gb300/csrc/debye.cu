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
#include <cmath>
#include <cstring>
#include <algorithm>
#include <vector>

#include "common.cuh"

using namespace bpmgb;

namespace {

constexpr int MAX_NA = 16;

struct NodeArgs {
  float alpha[MAX_NA];
  int n_ann;
  int steps;
};

struct DebyeLayout {
  size_t si, ct, wf, kr, trig, J, E, I, total;
  int T, M, Zo, nxo, nyo, nzo;
};

DebyeLayout debye_layout(const debye_desc* d) {
  DebyeLayout L;
  L.nxo = d->nx / 2 + 1;
  L.nyo = d->ny / 2 + 1;
  L.nzo = d->nz / 2 + 1;
  L.T = (d->n_na / 2) * (d->n_integration_steps + 1);
  L.M = L.nxo * L.nyo;
  L.Zo = L.nzo;
  size_t off = 0;
  L.si = off; off += align256(sizeof(double) * L.T);
  L.ct = off; off += align256(sizeof(double) * L.T);
  L.wf = off; off += align256(sizeof(float) * 3 * L.T);
  L.kr = off; off += align256(sizeof(double) * L.M);
  L.trig = off; off += align256(sizeof(float) * 4 * L.M);
  L.J = off; off += align256(sizeof(float) * 3 * (size_t)L.T * L.M);
  L.E = off; off += align256(sizeof(float2) * (size_t)L.T * L.Zo);
  L.I = off; off += align256(sizeof(float2) * 3 * (size_t)L.Zo * L.M);
  L.total = off;
  return L;
}

// x = x1 + i*(x2-x1)/(N-1.f) with x1 = 0, FP32 as the kernel evaluates it (psf_debye.cl:46-48)
__device__ __forceinline__ float coord_f32(int i, float x2, int N) {
  return 0.f + __fdiv_rn(__fmul_rn((float)i, x2 - 0.f), (float)N - 1.f);
}

// trapezoid nodes and weights per annulus (psf_debye.cl:62-78), FP64
__global__ void debye_nodes_kernel(NodeArgs a, double* si, double* ct, float* wf, int T) {
  int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= T) return;
  const int per = a.steps + 1;
  const int ann = idx / per, i = idx - ann * per;
  const double a1 = a.alpha[2 * ann], a2 = a.alpha[2 * ann + 1];
  const double dt = (a2 - a1) / (a.steps - 1.);
  const double t = a1 + i * dt;
  double s, c;
  sincos(t, &s, &c);
  const double w = ((i == 0 || i == a.steps) ? .5 : 1.) * dt * sqrt(c);
  si[idx] = s;
  ct[idx] = c;
  wf[idx] = (float)(w * (c + 1.));
  wf[T + idx] = (float)(w * s);
  wf[2 * T + idx] = (float)(w * (c - 1.));
}

// radius and azimuth per octant column (ix, jy)
__global__ void debye_radii_kernel(int nxo, int nyo, float x2, float y2, double k, double* kr, float* trig, int M) {
  int m = blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= M) return;
  const int jy = m / nxo, ix = m - jy * nxo;
  const double x = coord_f32(ix, x2, nxo), y = coord_f32(jy, y2, nyo);
  kr[m] = k * sqrt(x * x + y * y);
  const double phi = atan2(y, x);
  double s1, c1, s2, c2;
  sincos(phi, &s1, &c1);
  sincos(2. * phi, &s2, &c2);
  trig[m] = (float)c1;
  trig[M + m] = (float)s1;
  trig[2 * M + m] = (float)c2;
  trig[3 * M + m] = (float)s2;
}

// E(t, z) = exp(i kz cos t), phase formed and reduced in FP64
__global__ void debye_phase_kernel(int Zo, float z2, double k, const double* ct, float2* E, int T) {
  int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= T * Zo) return;
  const int t = idx / Zo, z = idx - t * Zo;
  const double kz = k * (double)coord_f32(z, z2, Zo);
  double s, c;
  sincos(kz * ct[t], &s, &c);
  E[idx] = make_float2((float)c, (float)s);
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
      term *= -q / (float)(k * (k + 2));
      sum += term;
    }
    return sum;
  }
  return 2.f * j1 / x - j0;
}

// A_n(t, m) = p_n(t) J_n(kr_m sin t_t)
__global__ void debye_bessel_kernel(int T, int M, const double* si, const double* kr, const float* wf, float* J) {
  const int m = blockIdx.x * blockDim.x + threadIdx.x;
  const int t = blockIdx.y;
  if (m >= M) return;
  const float x = (float)(kr[m] * si[t]);
  const float j0 = j0f(x), j1 = j1f(x);
  const float j2 = bessel_j2(x, j0, j1);
  const size_t TM = (size_t)T * M, o = (size_t)t * M + m;
  J[o] = wf[t] * j0;
  J[TM + o] = wf[T + t] * j1;
  J[2 * TM + o] = wf[2 * T + t] * j2;
}

// I_n(z, m) = sum_t A_n(t, m) E(t, z): tile of 64 radii x 32 planes per block, each thread
// owning 4 radii x 2 planes x 3 components.
constexpr int AM = 64, AZ = 32, AT = 16;

__global__ void __launch_bounds__(256) debye_accum_kernel(int T, int M, int Zo, const float* __restrict__ J,
                                                          const float2* __restrict__ E, float2* __restrict__ I) {
  __shared__ __align__(16) float Js[3][AT][AM];
  __shared__ __align__(16) float2 Es[AT][AZ];
  const int tid = threadIdx.x;
  const int tm = tid & 15, tz = tid >> 4;
  const int m0 = blockIdx.x * AM, z0 = blockIdx.y * AZ;
  float2 acc[3][4][2];
#pragma unroll
  for (int n = 0; n < 3; n++)
#pragma unroll
    for (int a = 0; a < 4; a++)
#pragma unroll
      for (int b = 0; b < 2; b++) acc[n][a][b] = make_float2(0.f, 0.f);
  const size_t TM = (size_t)T * M;
  for (int t0 = 0; t0 < T; t0 += AT) {
    for (int e = tid; e < 3 * AT * AM; e += 256) {
      const int n = e / (AT * AM), r = e - n * AT * AM;
      const int tt = r / AM, mm = r - tt * AM;
      const int t = t0 + tt, m = m0 + mm;
      Js[n][tt][mm] = (t < T && m < M) ? J[n * TM + (size_t)t * M + m] : 0.f;
    }
    for (int e = tid; e < AT * AZ; e += 256) {
      const int tt = e / AZ, zz = e - tt * AZ;
      const int t = t0 + tt, z = z0 + zz;
      Es[tt][zz] = (t < T && z < Zo) ? E[(size_t)t * Zo + z] : make_float2(0.f, 0.f);
    }
    __syncthreads();
#pragma unroll 4
    for (int tt = 0; tt < AT; tt++) {
      const float4 e4 = *reinterpret_cast<const float4*>(&Es[tt][tz * 2]);
      const float2 ev[2] = {make_float2(e4.x, e4.y), make_float2(e4.z, e4.w)};
#pragma unroll
      for (int n = 0; n < 3; n++) {
        const float4 j4 = *reinterpret_cast<const float4*>(&Js[n][tt][tm * 4]);
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
    __syncthreads();
  }
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

// full-volume assembly fused with the octant mirroring
__global__ void debye_assemble_kernel(int nx, int ny, int nz, int nxo, int M, int Zo, float ex0, float ey0,
                                      const float2* __restrict__ I, const float* __restrict__ trig,
                                      float* __restrict__ u, float2* __restrict__ ex, float2* __restrict__ ey,
                                      float2* __restrict__ ez) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y, z = blockIdx.z;
  if (x >= nx) return;
  const int ix = abs(x - nx / 2), jy = abs(y - ny / 2), kz = abs(z - nz / 2);
  const bool conj = z <= nz / 2;
  const int m = jy * nxo + ix;
  const size_t ZM = (size_t)Zo * M, o = (size_t)kz * M + m;
  const float2 I0 = __ldg(I + o), I1 = __ldg(I + ZM + o), I2 = __ldg(I + 2 * ZM + o);
  const float c1 = __ldg(trig + m), s1 = __ldg(trig + M + m);
  const float c2 = __ldg(trig + 2 * M + m), s2 = __ldg(trig + 3 * M + m);
  // psf_debye.cl:90-101
  float2 vx = make_float2(ex0 * (I0.x + I2.x * c2) + (ey0 * s2) * I2.x, ex0 * (I0.y + I2.y * c2) + (ey0 * s2) * I2.y);
  float2 vy = make_float2(ey0 * (I0.x - I2.x * c2) + (ex0 * s2) * I2.x, ey0 * (I0.y - I2.y * c2) + (ex0 * s2) * I2.y);
  const float pz = ex0 * c1 + ey0 * s1;
  float2 vz = make_float2(2.f * I1.y * pz, -2.f * I1.x * pz);
  const size_t v = ((size_t)z * ny + y) * nx + x;
  if (u) __stcs(u + v, cabs2(vx) + cabs2(vy) + cabs2(vz));
  if (conj) {
    vx.y = -vx.y;
    vy.y = -vy.y;
    vz.y = -vz.y;
  }
  if (ex) __stcs(ex + v, vx);
  if (ey) __stcs(ey + v, vy);
  if (ez) __stcs(ez + v, vz);
}

int check_desc(const debye_desc* d) {
  if (!d) { set_error("description is NULL"); return BPM_ERR_ARG; }
  if (d->nx < 2 || d->ny < 2 || d->nz < 2) { set_error("shape must be >= 2 in every axis"); return BPM_ERR_SHAPE; }
  if (d->nx % 2 + d->ny % 2 + d->nz % 2 != 0) {
    set_error("odd shapes not supported yet");  // _focus_fields_debye.py:81-82
    return BPM_ERR_SHAPE;
  }
  if (!d->na || d->n_na < 2 || d->n_na % 2 || d->n_na > MAX_NA) {
    set_error("NA must be a scalar or an even-length list of at most 16 values");
    return BPM_ERR_ARG;
  }
  if (d->n_integration_steps < 2) { set_error("n_integration_steps must be >= 2"); return BPM_ERR_ARG; }
  if (!(d->lam > 0) || !(d->n0 > 0) || !(d->dx > 0) || !(d->dy > 0) || !(d->dz >= 0)) {
    set_error("lam, n0, dx, dy must be positive and dz >= 0");
    return BPM_ERR_ARG;
  }
  return BPM_OK;
}

}  // namespace

extern "C" size_t debye_workspace_bytes(const debye_desc* d) {
  if (check_desc(d)) return 0;
  return debye_layout(d).total;
}

extern "C" int debye_focus_field(const debye_desc* d, float* u, void* ex, void* ey, void* ez, void* ws,
                                 size_t ws_bytes, void* stream) {
  clear_error();
  int rc = check_desc(d);
  if (rc) return rc;
  DebyeLayout L = debye_layout(d);
  if (!ws || ws_bytes < L.total) {
    set_error("workspace too small: need " + std::to_string(L.total) + " bytes");
    return BPM_ERR_OOM;
  }
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  char* w = static_cast<char*>(ws);
  double* si = reinterpret_cast<double*>(w + L.si);
  double* ct = reinterpret_cast<double*>(w + L.ct);
  float* wf = reinterpret_cast<float*>(w + L.wf);
  double* kr = reinterpret_cast<double*>(w + L.kr);
  float* trig = reinterpret_cast<float*>(w + L.trig);
  float* J = reinterpret_cast<float*>(w + L.J);
  float2* E = reinterpret_cast<float2*>(w + L.E);
  float2* I = reinterpret_cast<float2*>(w + L.I);

  // the float32 launch arguments of _focus_fields_debye.py:102-109
  NodeArgs na;
  memset(&na, 0, sizeof(na));
  na.n_ann = d->n_na / 2;
  na.steps = d->n_integration_steps;
  for (int i = 0; i < d->n_na; i++) na.alpha[i] = (float)asin(d->na[i] / d->n0);
  const float x2 = (float)(d->dx * (L.nxo - 1.)), y2 = (float)(d->dy * (L.nyo - 1.)),
              z2 = (float)(d->dz * (L.nzo - 1.));
  const float lamf = (float)(1. * d->lam / d->n0);
  const double k = 2. * M_PI / (double)lamf;

  debye_nodes_kernel<<<(L.T + 127) / 128, 128, 0, s>>>(na, si, ct, wf, L.T);
  BPM_LAUNCH_CHECK("debye_nodes_kernel");
  debye_radii_kernel<<<(L.M + 127) / 128, 128, 0, s>>>(L.nxo, L.nyo, x2, y2, k, kr, trig, L.M);
  BPM_LAUNCH_CHECK("debye_radii_kernel");
  debye_phase_kernel<<<(L.T * L.Zo + 127) / 128, 128, 0, s>>>(L.Zo, z2, k, ct, E, L.T);
  BPM_LAUNCH_CHECK("debye_phase_kernel");
  debye_bessel_kernel<<<dim3((L.M + 127) / 128, L.T), 128, 0, s>>>(L.T, L.M, si, kr, wf, J);
  BPM_LAUNCH_CHECK("debye_bessel_kernel");
  debye_accum_kernel<<<dim3((L.M + AM - 1) / AM, (L.Zo + AZ - 1) / AZ), 256, 0, s>>>(L.T, L.M, L.Zo, J, E, I);
  BPM_LAUNCH_CHECK("debye_accum_kernel");
  if (u || ex || ey || ez) {
    debye_assemble_kernel<<<dim3((d->nx + 127) / 128, d->ny, d->nz), 128, 0, s>>>(
        d->nx, d->ny, d->nz, L.nxo, L.M, L.Zo, (float)d->ex0, (float)d->ey0, I, trig, u,
        static_cast<float2*>(ex), static_cast<float2*>(ey), static_cast<float2*>(ez));
    BPM_LAUNCH_CHECK("debye_assemble_kernel");
  }
  return BPM_OK;
}
