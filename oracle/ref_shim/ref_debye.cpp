/*
 * Test infrastructure only (oracle). Compiles the reference's Debye-Wolf kernel
 * source bpm/psf/kernels/psf_debye.cl (which includes bessel.cl) from where it lies,
 * as host C++, and exposes a C ABI that runs one kernel launch as a loop over the
 * work-item grid. Used to pin the numpy restatement in oracle/debye_ref.py and to
 * generate golden vectors; never part of the product path.
 *
 * Launch being reproduced: bpm/psf/_focus_fields_debye.py:102-109 (global size =
 * octant shape (Nx, Ny, Nz)); INT_STEPS is the compile-time quadrature count of
 * psf_debye.cl:20-22, made a runtime variable here so one build serves every count.
 */
#include "cl_shim.h"

thread_local size_t shim_gid[3];
thread_local size_t shim_gsize[3];

static int shim_int_steps = 100;
#define INT_STEPS shim_int_steps

#undef M_PI
#include "psf_debye.cl"

extern "C" {

void ref_debye_wolf(cfloat_t* Ex, cfloat_t* Ey, cfloat_t* Ez, float* I,
                    float Ex0, float Ey0, float x1, float x2, float y1, float y2,
                    float z1, float z2, float lam, const float* alphas, int Nalphas,
                    int Nx, int Ny, int Nz, int int_steps) {
  shim_int_steps = int_steps;
#pragma omp parallel for schedule(dynamic, 1)
  for (int k = 0; k < Nz; k++) {
    shim_gsize[0] = Nx; shim_gsize[1] = Ny; shim_gsize[2] = Nz;
    for (int j = 0; j < Ny; j++) {
      for (int i = 0; i < Nx; i++) {
        shim_gid[0] = i; shim_gid[1] = j; shim_gid[2] = k;
        debye_wolf(Ex, Ey, Ez, I, Ex0, Ey0, x1, x2, y1, y2, z1, z2, lam, alphas, Nalphas);
      }
    }
  }
}

/* debye_wolf_plane (psf_debye.cl:117-183), launch _focus_fields_debye.py:201-209: (Nx, Ny) */
void ref_debye_wolf_plane(cfloat_t* Ex, float Ex0, float Ey0, float x1, float x2, float y1, float y2,
                          float z, float lam, const float* alphas, int Nalphas, int Nx, int Ny,
                          int int_steps) {
  shim_int_steps = int_steps;
#pragma omp parallel for schedule(dynamic, 1)
  for (int j = 0; j < Ny; j++) {
    shim_gsize[0] = Nx; shim_gsize[1] = Ny; shim_gsize[2] = 1;
    for (int i = 0; i < Nx; i++) {
      shim_gid[0] = i; shim_gid[1] = j; shim_gid[2] = 0;
      debye_wolf_plane(Ex, Ex0, Ey0, x1, x2, y1, y2, z, lam, alphas, Nalphas);
    }
  }
}

/* debye_wolf_at (psf_debye.cl:187-269), launch _focus_fields_debye.py:346-352: (N,) */
void ref_debye_wolf_at(const float* xs, const float* ys, const float* zs, cfloat_t* Ex, cfloat_t* Ey,
                       cfloat_t* Ez, float* I, float Ex0, float Ey0, float lam, const float* alphas,
                       int Nalphas, long N, int int_steps) {
  shim_int_steps = int_steps;
#pragma omp parallel for schedule(static)
  for (long i = 0; i < N; i++) {
    shim_gsize[0] = N; shim_gsize[1] = 1; shim_gsize[2] = 1;
    shim_gid[0] = i; shim_gid[1] = 0; shim_gid[2] = 0;
    debye_wolf_at(xs, ys, zs, Ex, Ey, Ez, I, Ex0, Ey0, lam, alphas, Nalphas);
  }
}

/* debye_wolf_gauss (psf_debye.cl:273-362), launch _focus_fields_debye.py:404-412: octant */
void ref_debye_wolf_gauss(cfloat_t* Ex, cfloat_t* Ey, cfloat_t* Ez, float* I, float Ex0, float Ey0,
                          float x1, float x2, float y1, float y2, float z1, float z2, float lam,
                          float sig, const float* alphas, int Nalphas, int Nx, int Ny, int Nz,
                          int int_steps) {
  shim_int_steps = int_steps;
#pragma omp parallel for schedule(dynamic, 1)
  for (int k = 0; k < Nz; k++) {
    shim_gsize[0] = Nx; shim_gsize[1] = Ny; shim_gsize[2] = Nz;
    for (int j = 0; j < Ny; j++) {
      for (int i = 0; i < Nx; i++) {
        shim_gid[0] = i; shim_gid[1] = j; shim_gid[2] = k;
        debye_wolf_gauss(Ex, Ey, Ez, I, Ex0, Ey0, x1, x2, y1, y2, z1, z2, lam, sig, alphas, Nalphas);
      }
    }
  }
}

void ref_bessel_jn(int n, const float* x, float* out, long count) {
  for (long i = 0; i < count; i++) out[i] = bessel_jn(n, x[i]);
}

}  /* extern "C" */
