/*
 * bpm_gb300 -- C ABI of the GB300 (sm_103a) implementation of bpm's two hot paths:
 *   (1) the split-step beam-propagation z-march (bpm_3d / Bpm3d), and
 *   (2) the vectorial Debye-Wolf focus field (focus_field_debye / psf / psf_u0).
 *
 * The reference (maweigert/bpm) has no C ABI: its boundary is the Python API, which
 * JIT-compiles OpenCL kernels and launches them through gputools/pyopencl. Each entry
 * point below replaces one such Python-level driver, cited per function. Buffers are
 * plain device pointers owned by the caller; the library allocates only plan-private
 * tables (at plan creation) and takes scratch from a caller-sized workspace.
 * All calls are stream-ordered on the `stream` argument (a cudaStream_t; NULL = legacy
 * default stream) and never synchronise the host, except plan creation, which uploads
 * its tables synchronously. A plan may be used from one host thread at a time.
 *
 * Arrays use the reference's layouts (numpy C order): a field plane is (ny, nx)
 * complex64 (interleaved float re, im), a volume (nz, ny, nx), a batch of fields
 * (batch, ny, nx); element (x, y, z) sits at x + nx*y + nx*ny*z.
 *
 * Return value: BPM_OK (0) or a negative bpm_status; bpm_last_error() gives the text
 * of the last error raised on the calling thread.
 */
#ifndef BPM_GB300_H
#define BPM_GB300_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define BPM_GB300_VERSION 1

typedef enum {
  BPM_OK = 0,
  BPM_ERR_ARG = -1,        /* invalid argument (the reference raises ValueError)            */
  BPM_ERR_SHAPE = -2,      /* unsupported shape (the reference raises NotImplementedError)  */
  BPM_ERR_OOM = -3,        /* device allocation failed or workspace too small               */
  BPM_ERR_CUDA = -4,       /* a CUDA runtime call failed                                    */
  BPM_ERR_TIMEOUT = -5,    /* a bounded device-side wait gave up                            */
  BPM_ERR_UNSUPPORTED = -6 /* combination the reference leaves undefined                    */
} bpm_status;

/* mean-index correction of the propagator, bpm/bpm/bpm_3d.py:53 mean_mode */
typedef enum {
  BPM_MEAN_IGNORE = 0,   /* fixed propagator at n0                                           */
  BPM_MEAN_SIMPLE = 1,   /* n0 + mean(dn[z]) per slice, given by the caller (slice tables)   */
  BPM_MEAN_WEIGHTED = 2  /* n0 + sum|u_hat|*dn0 / sum|u_hat| per step, reduced on the device */
} bpm_mean_mode;

/* which propagator recipe the plan reproduces */
typedef enum {
  BPM_PROP_FUNCTIONAL = 0, /* bpm_3d: FP32 FFTFREQ evanescent mask of compute_propagator
                              (bpm/bpm/kernels/bpm_3d_kernels.cl:408-432), FP64 kz phase  */
  BPM_PROP_CLASS = 1       /* Bpm3d: host FP64 propagator, NaN-mask (bpm/bpmclass/bpm3d.py:87-109) */
} bpm_prop_kind;

typedef enum {
  BPM_DN_NONE = 0,  /* free propagation, no phase mask and no taper                      */
  BPM_DN_F32 = 1,   /* real dn, float32                                                   */
  BPM_DN_F16 = 2,   /* real dn stored as IEEE half (store_dn_as_half)                     */
  BPM_DN_C64 = 3    /* complex dn, complex64: exp(-i k0 dz dn), no taper (reference Q7)  */
} bpm_dn_dtype;

typedef enum {
  BPM_OUT_NONE = 0,      /* no volume output (last plane only)                              */
  BPM_OUT_FIELD = 1,     /* complex64 field volume (return_field=True)                      */
  BPM_OUT_INTENSITY = 2  /* float32 |u|^2 volume (return_field=False)                       */
} bpm_out_kind;

typedef struct {
  int nx, ny, nz;          /* grid; nx, ny powers of two in [16, 1024]; nz >= 1              */
  double dx, dy, dz;       /* voxel size, microns                                            */
  double lam;              /* vacuum wavelength, microns                                     */
  double n0;               /* background refractive index                                    */
  int absorbing_width;     /* taper width in pixels (0 = none)                               */
  int mean_mode;           /* bpm_mean_mode                                                  */
  int prop_kind;           /* bpm_prop_kind                                                  */
  int use_fresnel_approx;  /* changes only the scattering weights (reference quirk Q1)       */
} bpm_grid_desc;

typedef struct bpm_plan bpm_plan;

/* One propagation request over `batch` fields that share the plan's grid. */
typedef struct {
  int batch;                     /* number of fields (>= 1)                                     */
  const void* u0;                /* device, (batch, ny, nx) complex64 input planes              */
  const void* dn;                /* device dn volume(s) of dtype dn_dtype, (nz, ny, nx) each    */
  int dn_dtype;                  /* bpm_dn_dtype                                                */
  long long dn_batch_stride;     /* elements between fields' dn volumes; 0 = one shared volume  */
  const float* slice_n;          /* BPM_MEAN_SIMPLE: device (nz) float32(n0 + mean(dn[z]))      */
  const float* slice_dn0;        /* BPM_MEAN_SIMPLE: device (nz) float32(mean(dn[z]))           */
  void* out;                     /* device output volume(s) of kind out_kind, or NULL           */
  int out_kind;                  /* bpm_out_kind                                                */
  long long out_batch_stride;    /* elements between fields' output volumes                     */
  void* last_plane;              /* device (batch, ny, nx) complex64 exit fields, or NULL       */
  float* scatter_p;              /* device (batch, nz) scattering cross-section, or NULL        */
  float* scatter_g;              /* device (batch, nz) anisotropy g (needs scatter_p), or NULL  */
  int scattering_plane_ind;      /* z offset of the plain-wave reference, bpm_3d.py:253         */
  int group;                     /* fields marched together per pass (0 = library default)      */
  void* ckpt;                    /* device (batch, (nz-1)/ckpt_every+1, ny, nx) complex64: the
                                    field at planes z = 0, k, 2k, ... (k = ckpt_every), or NULL  */
  int ckpt_every;                /* checkpoint spacing k (>= 1 when ckpt is set)                */
  const void* mask;              /* device (nz, ny, nx) complex64 phase masks of the shared dn
                                    from bpm_mask_precompute, or NULL to form them on the fly
                                    (results are bit-identical either way)                     */
  /* Launch shape (0 = the library's rule for each). None changes a result's bits, except
   * cluster at 64x64, where the two families run FFTs of another radix order (FP32 rounding). */
  int conc;                      /* groups marching at once on their own streams, 1..8
                                    (default BPM_GB300_CONC, else 4)                            */
  int col_block;                 /* columns per block of the non-weighted column passes, 4, 8 or 16 */
  int cluster;                   /* whole-march cluster kernel (square 64..256 grids without
                                    scattering sums or checkpoints): 1 = use it, 2 = row/column
                                    pass kernels (default: cluster at 64)                       */
  int col_fuse;                  /* weighted mode: 1 = one column pass per step (forward FFT,
                                    plane-wide sums across a thread-block cluster of the field's
                                    blocks, propagator, inverse FFT) where ny <= 512, nx <= 512
                                    and no scattering sums; 0 or 2 = the two column passes (the
                                    default; same bits either way)                               */
  int grad_sum;                  /* bpm_backward only: 1 = the fields share one dn volume
                                    (dn_batch_stride 0) and grad_dn is (nz, ny, nx), the dn
                                    gradient summed over the request's fields; 0 = per field   */
} bpm_request;

/* Library version (BPM_GB300_VERSION). */
int bpm_version(void);

/* Text of the last error on the calling thread ("" if none). */
const char* bpm_last_error(void);

/* Number of kernels this library has launched in the calling process (all threads). */
unsigned long long bpm_launch_count(void);

/* 1 if p is page-locked host memory that the current device reaches through the same
 * address (cudaHostAlloc / cudaHostRegister under unified addressing), else 0. Such a
 * buffer may be passed as bpm_request.out: the march then writes its output planes
 * straight into host memory over the CPU-GPU link, with no staging copy. (No reference
 * counterpart: the reference always reads its output back with a separate copy.) */
int bpm_host_ptr_mapped(const void* p);

/* Validate a grid description without touching the device (BPM_OK or an error). */
int bpm_grid_check(const bpm_grid_desc* desc);

/* Create a propagation plan: validates the grid and uploads the propagator, FFT twiddle,
 * taper and scattering-weight tables for the current device.
 * Replaces the setup half of bpm/bpm/bpm_3d.py:_bpm_3d (:140-278, propagator built by
 * compute_propagator at :192) and of bpm/bpmclass/bpm3d.py:_Bpm3d_Base._setup (:64-115)
 * + _bpm3d_ocl.py:_setup_impl (:35-56). */
int bpm_plan_create(const bpm_grid_desc* desc, bpm_plan** out);

/* A plan for the same grid with another number of planes nz, sharing the device tables
 * of `base` (none of them depends on nz): no device allocation and no synchronisation,
 * only the plan's own streams and events are created. `base` must outlive it. (No
 * reference counterpart: the reference rebuilds its propagator for every bpm_3d call.) */
int bpm_plan_derive(const bpm_plan* base, int nz, bpm_plan** out);

/* Release a plan: its streams and events, and its device tables unless it was derived. */
int bpm_plan_destroy(bpm_plan* plan);

/* Fields the march advances together per kernel launch for a request of `batch` fields
 * (req->group if set, else the library default; 0 for invalid arguments). */
int bpm_group_size(const bpm_plan* plan, int batch, int group);

/* Bytes of scratch bpm_propagate needs for a request of `batch` fields (256-aligned): one
 * slot per group of fields that may march at the same time (4 by default, 1..8 through the
 * environment variable BPM_GB300_CONC, each on its own stream forked from and joined back
 * to the caller's stream). Any workspace of at least one slot works; smaller ones march
 * the groups one after another. */
size_t bpm_workspace_bytes(const bpm_plan* plan, int batch, int group);

/* The same for `conc` groups marching at once (a request's conc; 0 = the default). */
size_t bpm_workspace_bytes_conc(const bpm_plan* plan, int batch, int group, int conc);

/* March every field of the request through all nz slices.
 * Replaces the hot loop of bpm/bpm/bpm_3d.py:_bpm_3d (:283-381, one fft / reduction /
 * mult_propagator* / fft / mult_dn* / copy_intens sequence per z-step) and of
 * bpm/bpmclass/_bpm3d_ocl.py:_propagate_single (:100-126), for `batch` fields at once.
 * Plane 0 of `out` is u0 (unmasked); plane z>0 is the field after step z-1 with the
 * mask of dn slice z (reference quirk Q8). */
int bpm_propagate(bpm_plan* plan, const bpm_request* req, void* workspace, size_t workspace_bytes,
                  void* stream);

/* bpm_propagate whose output volume also lands in host memory while the march runs:
 * req->out is the device volume; every time a group of fields has written another
 * chunk_planes planes, a plan-owned copy stream moves them to host_out (same layout and
 * element type as req->out: (batch, nz, ny, nx) with req->out_batch_stride). The copies
 * overlap the rest of the march; `stream` waits for the last one. host_out should be
 * page-locked for the copies to run asynchronously. Replaces the march + read-back of
 * bpm/bpm/bpm_3d.py:_bpm_3d (:283-381, then u_g.get() at :388-391), with the read-back
 * overlapped. */
int bpm_propagate_to_host(bpm_plan* plan, const bpm_request* req, void* host_out, int chunk_planes,
                          void* workspace, size_t workspace_bytes, void* stream);

/* Allocation-free march, for callers that may not allocate device memory where they
 * march (a host that gives this library a fixed device budget and forbids it cudaMalloc,
 * a plugin whose host owns all device memory, a latency-critical loop where cudaMalloc
 * would synchronise the device). Same request and results as bpm_propagate, but the
 * scratch is one fixed array of BPM_NOALLOC_SCRATCH_BYTES inside the library's device
 * image, held by every GPU that loads the library until the process exits. It allocates
 * nothing: no cudaMalloc, no cudaFree, no allocating library call. Fields are marched in
 * as many groups as the array needs. The limit is an area: one field's scratch, its plane
 * of nx*ny*8 bytes plus under 1 KiB of per-tile partial sums, must fit the array, so
 * nx*ny must stay below 2^20: every supported grid but 1024x1024 (1024x512 is accepted);
 * 1024x1024 is refused with BPM_ERR_OOM and a message naming the limit. The plan's device must be the current device (else
 * BPM_ERR_ARG). The first call on a device looks up the array's device address (with
 * that device current) and caches it; make that first call before any stream capture. All calls
 * share the one array: calls that can overlap on the GPU (different streams or threads)
 * race on it and must be serialised by the caller. Every byte of the array a call reads
 * was written earlier in the same call, so nothing needs clearing between calls.
 * No counterpart in the reference (which allocates its buffers per call through
 * OCLArray). */
#define BPM_NOALLOC_SCRATCH_BYTES (8u << 20)
int bpm_propagate_noalloc(bpm_plan* plan, const bpm_request* req, void* stream);

/* Kinds of pass for bpm_launch_pass. */
typedef enum {
  BPM_PASS_FIRST_ROW = 0,         /* plane 0 output + forward row FFT                         */
  BPM_PASS_COLUMN = 1,            /* column FFT, propagator, inverse column FFT (ignore/simple) */
  BPM_PASS_COLUMN_REDUCE = 2,     /* weighted: forward column FFT + |u_hat| partial sums      */
  BPM_PASS_COLUMN_PROPAGATE = 3,  /* weighted: propagator + inverse column FFT                */
  BPM_PASS_ROW = 4,               /* inverse row FFT, mask, plane z output, forward row FFT   */
  BPM_PASS_COLUMN_FUSED = 5       /* weighted: both column passes in one launch (col_fuse)    */
} bpm_pass_kind;

/* Launch exactly one pass of the march for the first group of fields of the request, for
 * step / plane index z, on `stream`. Used to time individual kernels (each pass is one
 * kernel launch); the passes in march order reproduce bpm_propagate. No reference
 * counterpart: the reference's per-step launches are the kernels of bpm_3d_kernels.cl. */
int bpm_launch_pass(bpm_plan* plan, const bpm_request* req, void* workspace, size_t workspace_bytes,
                    int pass, int z, void* stream);

/* Phase masks of a dn volume shared by many fields: mask[z][y][x] = taper * exp(-i k0 dz dn)
 * for real dn, exp(k0 dz Im dn) * exp(-i k0 dz Re dn) for complex dn (the factors of the
 * reference's mult_dn* kernels, bpm/bpm/kernels/bpm_3d_kernels.cl:20-283, without the
 * mean-index shift, which the march applies per field). Passing the result as req->mask
 * saves every field of a batch from re-evaluating them; (nz, ny, nx) complex64 output. */
int bpm_mask_precompute(bpm_plan* plan, const void* dn, int dn_dtype, void* mask, void* stream);

/* Capture the launches of bpm_propagate for a fixed request and workspace into a CUDA
 * graph; bpm_exec_launch replays it on any stream. The buffers named by `req` and the
 * workspace must stay valid and unchanged in address while the exec lives. No reference
 * counterpart (the reference re-enqueues every launch from Python each step). */
typedef struct bpm_exec bpm_exec;
int bpm_exec_create(bpm_plan* plan, const bpm_request* req, void* workspace, size_t workspace_bytes,
                    bpm_exec** out);
int bpm_exec_launch(bpm_exec* exec, void* stream);
int bpm_exec_destroy(bpm_exec* exec);

/* Bytes of scratch bpm_backward needs (256-aligned). */
size_t bpm_backward_workspace_bytes(const bpm_plan* plan, int batch, int group, int ckpt_every);

/* Adjoint of the march for mean_mode "ignore" with real (f32 / f16) or no dn: given
 * grad_last = dL/dRe(u_last) + i dL/dIm(u_last) for the exit planes, (batch, ny, nx)
 * complex64, write the gradient of L with respect to each field's dn into grad_dn
 * (batch, nz, ny, nx) float32 (plane z >= 1 written; plane 0 left untouched: plane 0 of
 * the march is u0, which dn does not reach) -- or, with req->grad_sum = 1 and one shared
 * dn, the gradient with respect to that dn, summed over the fields in a fixed order, into
 * grad_dn (nz, ny, nx) -- and, if grad_u0 is not NULL, the gradient
 * with respect to u0 into grad_u0 (batch, ny, nx) complex64. The request must be the one
 * the forward bpm_propagate ran with, including its checkpoints (req->ckpt,
 * req->ckpt_every): each segment between checkpoints is recomputed forward, then marched
 * backward with the conjugate propagator and conjugate phase masks.
 * No reference counterpart (the reference has no gradient; bpm/bpm/bpm_3d_inverse.py is a
 * non-functional sketch). */
int bpm_backward(bpm_plan* plan, const bpm_request* req, const void* grad_last, float* grad_dn,
                 void* grad_u0, void* workspace, size_t workspace_bytes, void* stream);

/* ---------------------------------------------------------------------------------- */
/* Coated-sphere refractive-index volumes                                              */
/* ---------------------------------------------------------------------------------- */

/* Fill dn (nz, ny, nx) float32 on the device with coated spheres: a voxel at
 * (dx*i, dy*j, dz*k) whose nearest centre lies within rad_inner gets dn_inner, within
 * rad_outer dn_outer, else 0. points: device (np, 3) float32 centres (x, y, z) in microns,
 * sorted by ascending z. Replaces bpm/bpm/bpm_3d_spheres.py:create_dn_buffer (:11-38) and
 * its kernel bpm/bpm/kernels/bpm_3d_spheres.cl:fill_dn (:31-74); bit-identical volume. */
int bpm_spheres_fill(int nx, int ny, int nz, double dx, double dy, double dz, const float* points, int np,
                     double dn_inner, double rad_inner, double dn_outer, double rad_outer, float* dn,
                     void* stream);

/* ---------------------------------------------------------------------------------- */
/* Vectorial Debye-Wolf focus field                                                    */
/* ---------------------------------------------------------------------------------- */

/* quadrature rule of debye_focus_field */
typedef enum {
  DEBYE_QUAD_REFERENCE = 0, /* the reference kernel's: INT_STEPS+1 nodes with dt = (a2-a1)/(INT_STEPS-1),
                               the last past a2, pupil factor sqrt(cos t) without sin t
                               (bpm/psf/kernels/psf_debye.cl:62-78)                              */
  DEBYE_QUAD_PHYSICAL = 1   /* the Debye integral's sqrt(cos t) sin t, exact trapezoid of INT_STEPS
                               nodes over [a1, a2] (the formula of the reference's
                               tests/test_psf_vectorial.py:15-42)                                */
} debye_quadrature;

typedef struct {
  int nx, ny, nz;            /* full output shape (even), arrays (nz, ny, nx)                  */
  double dx, dy, dz;         /* voxel size, microns                                            */
  double lam;                /* vacuum wavelength, microns                                     */
  double n0;                 /* refractive index of the immersion medium                      */
  const double* na;          /* host array of aperture NAs: [0, NA] or annuli [a1, a2, ...]     */
  int n_na;                  /* even, >= 2                                                     */
  int n_integration_steps;   /* INT_STEPS: the rule uses INT_STEPS+1 nodes per annulus         */
  double ex0, ey0;           /* input polarisation (the reference launches with 1, 0)          */
  int quadrature;            /* debye_quadrature (debye_focus_field only; 0 elsewhere)         */
} debye_desc;

/* Bytes of scratch debye_focus_field needs for this description (256-aligned). */
size_t debye_workspace_bytes(const debye_desc* desc);

/* Sticky device-side status of the tensor-core kernels: nonzero once one of their bounded
 * waits (an mbarrier that a TMA copy or a tensor-core product should complete) gave up
 * after 2 s, in which case that launch left its outputs unwritten. Synchronises with the
 * device to read it; clear != 0 resets it to 0. A negative bpm_status on a CUDA error.
 * No counterpart in the reference (its OpenCL kernels have no such waits). */
int bpm_device_status(int clear);

/* Self-test of those bounded waits: runs the tensor-core quadrature kernel once on a small
 * product whose loads announce more bytes than they deliver, so its waits give up after
 * wait_ms (0 < wait_ms <= 1000) and it leaves with the status set and its tensor memory
 * freed. Returns BPM_ERR_TIMEOUT when the waits gave up (the status is cleared again),
 * BPM_OK if the product completed, another negative status on a CUDA error. Allocates its
 * own small buffers and synchronises the device. No counterpart in the reference. */
int debye_tc_timeout_selftest(double wait_ms);

/* Compute the focus field on the full (nz, ny, nx) grid centred at index n/2.
 * Replaces bpm/psf/_focus_fields_debye.py:focus_field_debye (:48-146): the debye_wolf
 * octant launch (:102-109, kernel bpm/psf/kernels/psf_debye.cl:24-113) and the host-side
 * spreading of the octant to the full volume (:116-144), fused into device kernels. The
 * quadrature sums run as a 3xTF32 product on the tensor cores (tcgen05, TMA-staged
 * operands); BPM_GB300_DEBYE=fma selects FP32 FMA kernels (set before the first call).
 * u: float32 |E|^2 (may be NULL); ex, ey, ez: complex64 (each may be NULL). */
int debye_focus_field(const debye_desc* desc, float* u, void* ex, void* ey, void* ez,
                      void* workspace, size_t workspace_bytes, void* stream);

/* Bytes of scratch debye_focus_field_gauss needs (256-aligned); 0 for an invalid desc. */
size_t debye_gauss_workspace_bytes(const debye_desc* desc);

/* Focus field of a Gaussian-illuminated pupil, amplitude exp(-t^2/(2 alpha_max^2 sig^2)).
 * Replaces bpm/psf/_focus_fields_debye.py:focus_field_debye_gauss (:361-441) with the
 * kernel bpm/psf/kernels/psf_debye.cl:debye_wolf_gauss (:273-362), including its octant of
 * (N0+1)/2 samples per axis on [0, d*N] and its spreading without conjugation (:426-438).
 * Any shape >= 3 per axis. The reference's function has no n0 argument: pass n0 = 1 for
 * its behaviour (alphas = asin(na), wavelength lam). sig > 0. Outputs as debye_focus_field. */
int debye_focus_field_gauss(const debye_desc* desc, double sig, float* u, void* ex, void* ey,
                            void* ez, void* workspace, size_t workspace_bytes, void* stream);

/* Bytes of scratch debye_focus_field_plane / debye_focus_field_at need (256-aligned). */
size_t debye_points_workspace_bytes(const debye_desc* desc);

/* Ex on one plane at height z: (ny, nx) complex64 over x in [-(nx/2) dx, (nx - nx/2) dx]
 * (likewise y). Replaces bpm/psf/_focus_fields_debye.py:focus_field_debye_plane
 * (:149-214) with bpm/psf/kernels/psf_debye.cl:debye_wolf_plane (:117-183). nz and dz are
 * not used; nx, ny >= 2. */
int debye_focus_field_plane(const debye_desc* desc, double z, void* ex, void* workspace,
                            size_t workspace_bytes, void* stream);

/* Fields at n arbitrary points (device float32 arrays x, y, z, microns). u receives
 * |ex|^2, as the reference kernel writes it (psf_debye.cl:267); u, ex, ey, ez (complex64)
 * may each be NULL. Replaces bpm/psf/_focus_fields_debye.py:focus_field_debye_at
 * (:315-358) with bpm/psf/kernels/psf_debye.cl:debye_wolf_at (:187-269). Only the optical
 * fields of desc (lam, n0, na, n_integration_steps, ex0, ey0) are used. */
int debye_focus_field_at(const debye_desc* desc, const float* x, const float* y, const float* z,
                         long long n, float* u, void* ex, void* ey, void* ez, void* workspace,
                         size_t workspace_bytes, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* BPM_GB300_H */
