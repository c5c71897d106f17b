/*
 * monte.h -- C ABI of libmonte, the GB300 (sm_103a) implementation of the
 * two data-parallel hot paths of the Monte CBCT code:
 *
 *   - FDK reconstruction: cosine weighting, Ram-Lak ramp filter and
 *     voxel-driven cone-beam backprojection (reference: recon/bp3d20.cpp,
 *     recon/bp3d20_325.cpp), plus the exact adjoint of the backprojector.
 *   - Photon-history Monte Carlo: Woodcock tracking through a label volume,
 *     photoelectric / Rayleigh / Klein-Nishina Compton interactions from the
 *     XCOM tables and the detector tally (reference: monte_cu/CBCT_real325im.cu,
 *     monte_cu/CBCT_real325.cu, monte_cpp/CBCT_real2.cpp).
 *
 * Conventions
 *   - Every entry point returns MONTE_OK (0) or a negative MONTE_E* code and
 *     never exits the process; monte_last_error() gives the text.
 *   - Pointers are caller-owned.  The `mem` argument of a call says whether
 *     its array arguments live in device memory (MONTE_MEM_DEVICE) or host
 *     memory (MONTE_MEM_HOST).  With host memory the library stages the data
 *     through device buffers it owns and copies results back before returning.
 *   - One context per host thread; a context owns one CUDA stream.  Device
 *     calls are asynchronous on that stream unless `mem` is MONTE_MEM_HOST.
 *   - There is no CPU fallback: without a usable GPU every compute call fails
 *     with MONTE_ECUDA.
 *
 * Units are the reference's: centimetres, keV, g/cm^3, cm^2/g.
 */
#ifndef MONTE_H
#define MONTE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MONTE_ABI_VERSION 1

/* ---- status codes --------------------------------------------------- */
#define MONTE_OK            0
#define MONTE_EINVAL       -1  /* bad argument (null pointer, size, enum) */
#define MONTE_ENOMEM       -2  /* device or host allocation failed */
#define MONTE_ECUDA        -3  /* CUDA runtime/driver error, or no usable GPU */
#define MONTE_ETIMEOUT     -4  /* a bounded device wait gave up */
#define MONTE_EUNSUPPORTED -5  /* valid request this build/GPU cannot run */
#define MONTE_EOVERFLOW    -6  /* sizes overflow the index types */

#define MONTE_MEM_DEVICE 0
#define MONTE_MEM_HOST   1

typedef struct monte_ctx monte_ctx;

/* ---- context ---------------------------------------------------------- */
/* Version of this ABI (MONTE_ABI_VERSION). */
int monte_abi_version(void);
/* Create a context on CUDA device `device` with its own non-blocking stream. */
int monte_ctx_create(monte_ctx** out, int device);
int monte_ctx_destroy(monte_ctx* ctx);
/* Text of the last error raised on `ctx` (or of the last failed
 * monte_ctx_create when ctx is NULL). Never NULL. */
const char* monte_last_error(const monte_ctx* ctx);
/* Use a caller-provided cudaStream_t (NULL restores the context's own). */
int monte_ctx_set_stream(monte_ctx* ctx, void* cuda_stream);
/* Wait for all work queued on the context's stream. */
int monte_ctx_synchronize(monte_ctx* ctx);

/* ======================================================================
 *  FDK
 * ====================================================================== */

/* Quirk switches of the reference FDK programs (both on in
 * monte_fdk_geom_reference65/325). */
#define MONTE_FDK_TAN_DEGREES 0x1 /* BP distance term evaluates tan() of the view
                                     angle in degrees as if radians
                                     (recon/bp3d20.cpp:137) */
#define MONTE_FDK_FLAT_EDGE   0x2 /* bilinear neighbours past the last detector
                                     column/row read the flat array onward (next
                                     row / next view), zero past its end
                                     (recon/bp3d20.cpp:152-158) */

/*
 * Geometry of one FDK reconstruction.  Replaces the hard-coded constants of
 * recon/bp3d20.cpp:17-19,40,48-60,85-161 and recon/bp3d20_325.cpp:17-18,43,
 * 97-171.
 *
 * Projections are read as proj[view][u][v] (u: in-plane detector index, the
 * filter axis; v: axial index), recon/bp3d20.cpp:28-40.  The filtered
 * projections are written transposed, filtered[view][v][u]
 * (recon/bp3d20.cpp:70).  Detector index a sits at u = half_u - du*a, index b
 * at v = half_v - dv*b.  View k is at beta_k = k*360/n_views degrees.
 * Voxel (s,t,z) is at X = x0 + dvox*s, Y = y0 - dvox*t, Z = z0 - dvox*z;
 * outputs vol_xy[z][t][s] and vol_zy[s][t][z] (recon/bp3d20.cpp:160-161).
 */
typedef struct monte_fdk_geom {
  int32_t n_views;        /* projections over 360 degrees */
  int32_t nu;             /* detector columns (in-plane, filter axis) */
  int32_t nv;             /* detector rows (axial) */
  int32_t flags;          /* MONTE_FDK_* */
  double du, dv;          /* detector pitch (cm) */
  double half_u, half_v;  /* detector half extents (cm) */
  double sod;             /* source to rotation axis (cm) */
  double sdd;             /* source to detector plane (cm) */
  double wdist;           /* D of the cosine weight D/sqrt(D^2+u^2+v^2) and of
                             the distance weight D^2/(D-d)^2 */
  int32_t nx, ny, nz;     /* output grid (s, t, z) */
  int32_t s_begin, s_end; /* reconstructed s range [s_begin, s_end) */
  double dvox;            /* voxel pitch (cm) */
  double x0, y0, z0;      /* voxel origin, see above */
  int32_t mask_radius;    /* >0: only voxels with (s-nx/2)^2+(t-ny/2)^2+(z-nz/2)^2
                             <= mask_radius^2 are reconstructed */
  int32_t reserved0;
  double scale;           /* output = bp * scale * scale2 */
  double scale2;          /* second factor, applied after `scale` */
} monte_fdk_geom;

/* Filter implementations. */
#define MONTE_FILTER_FP32   0  /* FP32 CUDA-core Toeplitz GEMM */
#define MONTE_FILTER_BF16X3 1  /* tcgen05 tensor cores, split 3xBF16, FP32 accumulate */
/* Backprojector implementations. */
#define MONTE_BP_PLAIN 0  /* one voxel per thread, projections through L1/L2 */
#define MONTE_BP_TILED 1  /* TMA-staged shared-memory projection tiles, several
                             z-voxels per thread */

/* Defaults equal to recon/bp3d20.cpp (65x65 detector, 0.5 cm pitch,
 * 256^3 grid, slab s in [125,130), sphere mask 118, scale 2.7). */
void monte_fdk_geom_reference65(monte_fdk_geom* g);
/* Defaults equal to recon/bp3d20_325.cpp (325x325 detector, 0.1 cm pitch,
 * no mask, scale 2.7 then 5). */
void monte_fdk_geom_reference325(monte_fdk_geom* g);

/* Cosine weighting + ramp filter: proj[view][u][v] -> filtered[view][v][u].
 * recon/bp3d20.cpp:36-73. */
int monte_fdk_filter(monte_ctx* ctx, const monte_fdk_geom* g, const float* proj,
                     float* filtered, int filter_mode, int mem);
/* Voxel-driven backprojection of filtered[view][v][u] into vol_xy[nz][ny][nx]
 * (overwritten; voxels outside the slab/mask are set to 0) and, if not NULL,
 * vol_zy[nx][ny][nz].  recon/bp3d20.cpp:81-166. */
int monte_fdk_backproject(monte_ctx* ctx, const monte_fdk_geom* g, const float* filtered,
                          float* vol_xy, float* vol_zy, int bp_mode, int mem);
/* Full FDK: filter then backproject.  `filtered` may be NULL (device scratch
 * owned by the context is used instead).  recon/bp3d20.cpp:15-194. */
int monte_fdk(monte_ctx* ctx, const monte_fdk_geom* g, const float* proj, float* filtered,
              float* vol_xy, float* vol_zy, int filter_mode, int bp_mode, int mem);

#ifdef __cplusplus
}
#endif
#endif /* MONTE_H */
