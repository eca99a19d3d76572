/*
 * Test infrastructure only (oracle). Compiles the reference's elementwise BPM kernel
 * source bpm/bpm/kernels/bpm_3d_kernels.cl from where it lies, as host C++, and
 * exposes each kernel used by the split-step march (bpm/bpm/bpm_3d.py:192-381) as a
 * C function that runs one launch as a loop over the work-item grid. Together with
 * an FFT from numpy/scipy this reproduces the reference's per-step arithmetic
 * (propagator, evanescent mask, phase masks with taper, intensity copy) bit for bit
 * where no FFT is involved. Never part of the product path.
 */
#include "cl_shim.h"

#undef M_PI
#include "bpm_3d_kernels.cl"

#define SHIM_GRID2(NX, NY, CALL)                                   \
  for (int j = 0; j < (NY); j++) {                                 \
    for (int i = 0; i < (NX); i++) {                               \
      shim_gsize[0] = (NX); shim_gsize[1] = (NY); shim_gsize[2] = 1; \
      shim_gid[0] = i; shim_gid[1] = j; shim_gid[2] = 0;           \
      CALL;                                                        \
    }                                                              \
  }

#define SHIM_GRID1(N, CALL)                                        \
  for (int i = 0; i < (N); i++) {                                  \
    shim_gsize[0] = (N); shim_gsize[1] = 1; shim_gsize[2] = 1;     \
    shim_gid[0] = i; shim_gid[1] = 0; shim_gid[2] = 0;             \
    CALL;                                                          \
  }

extern "C" {

/* bpm_3d_kernels.cl:408 compute_propagator, launched (Nx, Ny) at bpm_3d.py:192 */
void ref_compute_propagator(cfloat_t* H, float n0, float k0, float dx, float dy, float dz,
                            int Nx, int Ny) {
  SHIM_GRID2(Nx, Ny, compute_propagator(H, n0, k0, dx, dy, dz));
}

/* bpm_3d_kernels.cl:437 mult_propagator (mean_mode="simple", bpm_3d.py:289) */
void ref_mult_propagator(cfloat_t* plane, float n0, float k0, float dx, float dy, float dz,
                         int Nx, int Ny) {
  SHIM_GRID2(Nx, Ny, mult_propagator(plane, n0, k0, dx, dy, dz));
}

/* bpm_3d_kernels.cl:465 mult_propagator_buff (mean_mode="weighted", bpm_3d.py:305) */
void ref_mult_propagator_buff(cfloat_t* plane, float* dn_sum, float* u_sum, float n00,
                              float k0, float dx, float dy, float dz, int Nx, int Ny) {
  SHIM_GRID2(Nx, Ny, mult_propagator_buff(plane, dn_sum, u_sum, n00, k0, dx, dy, dz));
}

/* bpm_3d_kernels.cl:11 mult (mean_mode="ignore", bpm_3d.py:314; Bpm3d, _bpm3d_ocl.py:103) */
void ref_mult(cfloat_t* a, cfloat_t* b, int N) { SHIM_GRID1(N, mult(a, b)); }

/* bpm_3d_kernels.cl:20 mult_dn (Bpm3d class path, _bpm3d_ocl.py:115) */
void ref_mult_dn(cfloat_t* input, float* dn, float unit_k, int stride, int absorb, int Nx, int Ny) {
  SHIM_GRID2(Nx, Ny, mult_dn(input, dn, unit_k, stride, absorb));
}
void ref_mult_dn_half(cfloat_t* input, half* dn, float unit_k, int stride, int absorb, int Nx, int Ny) {
  SHIM_GRID2(Nx, Ny, mult_dn_half(input, dn, unit_k, stride, absorb));
}
void ref_mult_dn_complex(cfloat_t* input, cfloat_t* dn, float unit_k, int stride, int absorb,
                         int Nx, int Ny) {
  SHIM_GRID2(Nx, Ny, mult_dn_complex(input, dn, unit_k, stride, absorb));
}

/* bpm_3d_kernels.cl:198/232/265 mult_dn_mean* (simple/ignore modes, bpm_3d.py:366-371) */
void ref_mult_dn_mean(cfloat_t* input, float* dn, float unit_k, float dn0, int stride, int absorb,
                      int Nx, int Ny) {
  SHIM_GRID2(Nx, Ny, mult_dn_mean(input, dn, unit_k, dn0, stride, absorb));
}
void ref_mult_dn_mean_half(cfloat_t* input, half* dn, float unit_k, float dn0, int stride,
                           int absorb, int Nx, int Ny) {
  SHIM_GRID2(Nx, Ny, mult_dn_mean_half(input, dn, unit_k, dn0, stride, absorb));
}
void ref_mult_dn_mean_complex(cfloat_t* input, cfloat_t* dn, float unit_k, cfloat_t dn0, int stride,
                              int absorb, int Nx, int Ny) {
  SHIM_GRID2(Nx, Ny, mult_dn_mean_complex(input, dn, unit_k, dn0, stride, absorb));
}

/* bpm_3d_kernels.cl:104/139 mult_dn_mean*_buff (weighted mode, bpm_3d.py:355-363) */
void ref_mult_dn_mean_buff(cfloat_t* input, float* dn, float* dn_sum, float* u_sum, float unit_k,
                           int stride, int absorb, int Nx, int Ny) {
  SHIM_GRID2(Nx, Ny, mult_dn_mean_buff(input, dn, dn_sum, u_sum, unit_k, stride, absorb));
}
void ref_mult_dn_mean_half_buff(cfloat_t* input, half* dn, float* dn_sum, float* u_sum,
                                float unit_k, int stride, int absorb, int Nx, int Ny) {
  SHIM_GRID2(Nx, Ny, mult_dn_mean_half_buff(input, dn, dn_sum, u_sum, unit_k, stride, absorb));
}

/* bpm_3d_kernels.cl:396 copy_intens (return_field=False, bpm_3d.py:274, :380) */
void ref_copy_intens(cfloat_t* plane, float* output, int stride, int N) {
  SHIM_GRID1(N, copy_intens(plane, output, stride));
}

}  /* extern "C" */
