// On-device coated-sphere refractive-index volumes.
//
// Reference: bpm/bpm/bpm_3d_spheres.py:create_dn_buffer (:11-38) launches
// bpm/bpm/kernels/bpm_3d_spheres.cl:fill_dn (:31-74) over (Nx, Ny, Nz): every voxel at
// r = (dx*i, dy*j, dz*k) finds the z-sorted sphere centres within rad_outer of its z plane,
// takes the smallest distance d to them and sets dn = dn_inner if d < rad_inner, dn_outer
// if d < rad_outer, 0 otherwise. Here the candidate range comes from two binary searches
// over the sorted z column instead of the reference's linear scans from both ends (same
// indices), and the distances are FP32 with every operation rounded as written, as the
// reference kernel evaluates them, so the volume is bit-identical. Generating the volume on
// the device saves the host->device upload of dn for served requests.
#include "common.cuh"

using namespace bpmgb;

namespace {

__global__ void spheres_fill_kernel(float* __restrict__ dn, const float* __restrict__ pts, int np, float dx, float dy,
                                    float dz, float dn1, float rad1, float dn2, float rad2, int nx, int ny) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y, k = blockIdx.z;
  if (i >= nx) return;
  const float rx = __fmul_rn(dx, (float)i), ry = __fmul_rn(dy, (float)j), rz = __fmul_rn(dz, (float)k);
  const float lo = __fsub_rn(rz, rad2), hi = __fadd_rn(rz, rad2);
  // ind1: first centre with z >= lo, at most np-1 (fill_dn's forward scan)
  int a = 0, b = np - 1;
  while (a < b) {
    const int m = (a + b) >> 1;
    if (__ldg(pts + 3 * m + 2) < lo) a = m + 1; else b = m;
  }
  const int ind1 = a;
  // ind2: last centre with z <= hi, at least 0 (fill_dn's backward scan)
  a = 0;
  b = np - 1;
  while (a < b) {
    const int m = (a + b + 1) >> 1;
    if (__ldg(pts + 3 * m + 2) > hi) b = m - 1; else a = m;
  }
  const int ind2 = a;
  float dmin = __fmul_rn(1000000000.f, rad2);
  for (int n = ind1; n <= ind2; n++) {
    const float ex = __fsub_rn(rx, __ldg(pts + 3 * n)), ey = __fsub_rn(ry, __ldg(pts + 3 * n + 1)),
                ez = __fsub_rn(rz, __ldg(pts + 3 * n + 2));
    float s = __fmul_rn(ex, ex);
    s = __fadd_rn(s, __fmul_rn(ey, ey));
    s = __fadd_rn(s, __fmul_rn(ez, ez));
    const float d = __fsqrt_rn(s);
    dmin = (d < dmin) ? d : dmin;
  }
  dn[((size_t)k * ny + j) * nx + i] = (dmin < rad2) ? ((dmin < rad1) ? dn1 : dn2) : 0.f;
}

}  // namespace

extern "C" int bpm_spheres_fill(int nx, int ny, int nz, double dx, double dy, double dz, const float* points, int np,
                                double dn_inner, double rad_inner, double dn_outer, double rad_outer, float* dn,
                                void* stream) {
  clear_error();
  if (nx < 1 || ny < 1 || nz < 1 || ny > 65535 || nz > 65535) { set_error("bad volume shape"); return BPM_ERR_SHAPE; }
  if (np < 1 || !points || !dn) { set_error("points (np >= 1) and dn must be given"); return BPM_ERR_ARG; }
  dim3 g((nx + 127) / 128, ny, nz);
  spheres_fill_kernel<<<g, 128, 0, static_cast<cudaStream_t>(stream)>>>(
      dn, points, np, (float)dx, (float)dy, (float)dz, (float)dn_inner, (float)rad_inner, (float)dn_outer,
      (float)rad_outer, nx, ny);
  BPM_LAUNCH_CHECK("spheres_fill_kernel");
  return BPM_OK;
}
