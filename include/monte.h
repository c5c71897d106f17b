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
 *   - A context keeps grow-only device buffers until it is destroyed:
 *     staging and scratch arrays, per-geometry tables, and the tiled
 *     backprojector's footprint table of its last geometry (4 bytes per
 *     block of voxel columns and view, at most 256 MB).
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
/* Queue the context's work on a caller-provided cudaStream_t; NULL means
 * the CUDA legacy default stream (stream 0).  A switch first waits for the
 * work the context queued on its current stream (its buffers are reused by
 * the next call), so that stream must still exist; the new one must stay
 * valid while the context uses it. */
int monte_ctx_set_stream(monte_ctx* ctx, void* cuda_stream);
/* Go back to the context's own non-blocking stream (waiting as above). */
int monte_ctx_use_own_stream(monte_ctx* ctx);
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
 * recon/bp3d20.cpp:36-73.  With MONTE_MEM_HOST and both buffers pinned the
 * views go up, through the filter and back down in overlapping ranges. */
int monte_fdk_filter(monte_ctx* ctx, const monte_fdk_geom* g, const float* proj,
                     float* filtered, int filter_mode, int mem);
/* Voxel-driven backprojection of filtered[view][v][u] into vol_xy[nz][ny][nx]
 * (overwritten; voxels outside the slab/mask are set to 0) and, if not NULL,
 * vol_zy[nx][ny][nz].  recon/bp3d20.cpp:81-166.  With MONTE_MEM_HOST,
 * MONTE_BP_TILED, a full-width volume and pinned buffers, the views are
 * uploaded in ranges under the backprojection of the earlier ranges, as in
 * monte_fdk. */
int monte_fdk_backproject(monte_ctx* ctx, const monte_fdk_geom* g, const float* filtered,
                          float* vol_xy, float* vol_zy, int bp_mode, int mem);
/* Full FDK: filter then backproject.  `filtered` may be NULL (device scratch
 * owned by the context is used instead).  recon/bp3d20.cpp:15-194.
 * With MONTE_MEM_HOST, MONTE_BP_TILED, a full-width volume (s_begin 0,
 * s_end nx) and every host buffer pinned (cudaHostAlloc / cudaHostRegister),
 * the call is pipelined: the views are uploaded in ranges on a copy stream,
 * each range filtered as it lands and backprojected into running sums, and
 * the last range writes the volume straight into the pinned buffers.  The
 * results equal the unpipelined path's bit for bit. */
int monte_fdk(monte_ctx* ctx, const monte_fdk_geom* g, const float* proj, float* filtered,
              float* vol_xy, float* vol_zy, int filter_mode, int bp_mode, int mem);
/* View ranges of the last host-memory monte_fdk, monte_fdk_filter or
 * monte_fdk_backproject call of this context: >= 1 when it ran pipelined,
 * 0 when it ran unpipelined. */
int monte_fdk_last_host_ranges(const monte_ctx* ctx);

/* Exact adjoint of monte_fdk_backproject (MONTE_BP_PLAIN coefficients): the
 * ray-driven cone-beam forward projector, vol_xy[nz][ny][nx] ->
 * filtered_out[view][v][u] (overwritten).  Needs flags without
 * MONTE_FDK_FLAT_EDGE (MONTE_EUNSUPPORTED otherwise).  No counterpart in
 * the reference; the transpose of recon/bp3d20.cpp:81-166. */
int monte_fdk_forward_project(monte_ctx* ctx, const monte_fdk_geom* g, const float* vol_xy,
                              float* filtered_out, int mem);
/* Adjoint of the whole FDK (monte_fdk with MONTE_FILTER_FP32 and
 * MONTE_BP_PLAIN): grad_proj[view][u][v] = W * T^T * A^T grad_vol, the
 * gradient of <grad_vol, FDK(proj)> with respect to proj.  Same flag
 * condition as monte_fdk_forward_project. */
int monte_fdk_backward(monte_ctx* ctx, const monte_fdk_geom* g, const float* grad_vol,
                       float* grad_proj, int mem);

/* Backprojection autotuner (no counterpart in the reference, whose
 * backprojection is a fixed CPU loop nest, recon/bp3d20.cpp:83-166): times
 * every tile shape (voxels per thread along z, columns per CTA, views per
 * shared-memory stage) of MONTE_BP_TILED on geometry g and makes the fastest
 * the context's choice for MONTE_BP_TILED.  *best receives its index, or -1
 * if no tile shape fits g (MONTE_BP_TILED then runs the plain kernel). */
int monte_fdk_autotune(monte_ctx* ctx, const monte_fdk_geom* g, int* best);
/* Choose the tile shape MONTE_BP_TILED uses on this context (-1: the
 * default shape); a shape that does not fit a geometry falls back to the
 * default, then to the plain kernel. */
int monte_fdk_set_bp_variant(monte_ctx* ctx, int variant);
/* Which kernel the last monte_fdk_backproject/monte_fdk call of this context
 * ran: a tile shape index >= 0, or -1 for MONTE_BP_PLAIN. */
int monte_fdk_last_bp_variant(const monte_ctx* ctx);
/* How often the tiled backprojectors left FP32 since the last reset:
 * counts[0] = voxel-view pairs decided in double next to a discontinuity
 * of the reference operator (the detector edges, recon/bp3d20.cpp:116,152),
 * counts[1] = (voxel column, view) pairs whose distance-weight sign was
 * taken in double (tmp_s near 0, :140).  Waits for the context's stream;
 * reset != 0 zeroes the counters.  No counterpart in the reference: it
 * bounds the double-precision share of a run. */
int monte_fdk_exact_counts(monte_ctx* ctx, uint64_t* counts, int reset);
/* Check the context's status word: MONTE_ETIMEOUT if a bounded wait inside
 * a kernel gave up since the last check (the word is then cleared).
 * Synchronizes the context's stream. */
int monte_ctx_check_status(monte_ctx* ctx);

/* ======================================================================
 *  2-D fan-beam FBP
 * ====================================================================== */

/*
 * Geometry of the reference's 2-D fan-beam FBP, recon/fbp2.cpp: n_det
 * detector elements at `pitch` (element c at u = -half + pitch*c, the
 * weighting's convention, :36-40), views k*360/n_views degrees, of which
 * [view_begin, view_end) are backprojected (the reference skips view 0,
 * :89); pixel (s, t) of the nx x ny image at X = x0 + pix*s, Y = y0 - pix*t;
 * the nearest detector element int((half - u') / pitch) is read (no
 * interpolation, :120-126); output image[t][s] += (D^2/(D-d)^2) * q * dbeta
 * * scale (:148).  Flag MONTE_FDK_TAN_DEGREES: tan() of the view angle in
 * degrees (as the reference evaluates it, :135).
 */
typedef struct monte_fbp2_geom {
  int32_t n_views, n_det;
  int32_t view_begin, view_end;
  int32_t nx, ny;
  int32_t flags;              /* MONTE_FDK_TAN_DEGREES */
  int32_t reserved0;
  double pitch, half;         /* detector pitch and half extent (cm) */
  double sod, sdd;            /* source to axis, source to detector (cm) */
  double wdist;               /* D of the weights */
  double pix, x0, y0;         /* image pitch and origin (cm) */
  double scale;
} monte_fbp2_geom;

/* Defaults equal to recon/fbp2.cpp: 65 elements of 0.5 cm, 360 views of
 * which 1..359 are backprojected, SOD 160, SDD 220, D 60, 256^2 image at
 * 0.1 cm from (-12.8, 12.8), scale 1.7, tan of degrees. */
void monte_fbp2_geom_reference(monte_fbp2_geom* g);

/* Weighting + ramp filter + backprojection: proj[view][det] ->
 * filtered[view][det] (may be NULL) and image[ny][nx] (overwritten).
 * recon/fbp2.cpp:15-152.  Double arithmetic as the reference's; the
 * filtered array and the image are float as there.  The call waits for the
 * context's stream (its per-view tables are staged from the host). */
int monte_fbp2(monte_ctx* ctx, const monte_fbp2_geom* g, const float* proj, float* filtered,
               float* image, int mem);

/* ======================================================================
 *  Monte Carlo
 * ====================================================================== */

/* Physics switches reproducing the reference programs' behaviour. */
#define MONTE_MC_STALE_SIN_PHI     0x1 /* a 2nd or later Compton rotates from the
                                          emission sin_phi_a, which the GPU program
                                          never refreshes (monte_cu/CBCT_real325im.cu:768-773) */
#define MONTE_MC_FIRST_COMPTON_Z   0x2 /* the first Compton turns about +z: the CPU
                                          program starts from sin_theta_a_new = 0
                                          (monte_cpp/CBCT_real2.cpp:193,460-463) */
#define MONTE_MC_NO_RAYLEIGH_TALLY 0x4 /* photons whose last interaction was Rayleigh
                                          are not tallied (monte_cpp/CBCT_real2.cpp:373-397) */
/* Transport switch (not a reference behaviour): delta tracking against
 * majorants local to macro cells of the phantom -- per cell, the largest
 * attenuation among the labels of the cell and its 26 neighbours, under
 * which a photon moves as far as no larger attenuation lies -- instead of
 * the reference's single majorant over the whole phantom
 * (monte_cu/CBCT_real325im.cu:866-868).  Exact in distribution -- the same
 * tallies in expectation -- but the random numbers are used differently,
 * so histories differ from those without the flag.  Far fewer virtual
 * collisions where soft tissue or air neighbours bone.  The macro cells are
 * 2^k voxels on a side, the smallest power of two >= 2 that leaves at most
 * 96 cells along the longest axis.  A context keeps the tables of its last
 * phantom and reuses them while the grid, the materials and the labels are
 * unchanged; with device labels it keeps a copy of the label volume
 * (nx*ny*nz bytes of device memory) and compares it on the device at each
 * call.  Not supported by monte_mc_run_noalloc. */
#define MONTE_MC_LOCAL_MAJORANT    0x8

/* Kernels. */
#define MONTE_MC_PLAIN      0 /* one thread per emitting pixel, histories in sequence
                                 (the reference's launch shape, CBCT_real325im.cu:462-464) */
#define MONTE_MC_PERSISTENT 1 /* persistent warps that refill lanes as histories end */

/*
 * Acquisition geometry of the Monte Carlo.  Replaces the #defines and
 * constants of monte_cu/CBCT_real325im.cu:6-18,459-460 and
 * monte_cpp/CBCT_real2.cpp:8-9,205-254.  The source sits at (-sod, 0, 0)
 * rotated by the view angle k*360/n_views degrees about z; the detector
 * plane is at distance sdd from the source.  Pixel (i, j) of a view is
 * centred at u = half_u - du*(i+0.5) (in-plane) and v = half_v - dv*(j+0.5)
 * (axial); every history of pixel (i, j) is aimed at that centre
 * (CBCT_real325im.cu:476-512).  Photons start on the plane x' = -start_plane
 * of the view frame (:522-540).
 */
typedef struct monte_mc_geom {
  int32_t n_views;
  int32_t nu, nv;           /* detector pixels (in-plane, axial) */
  int32_t max_interactions; /* interactions followed per history (ScatterNUM) */
  uint32_t flags;           /* MONTE_MC_* */
  int32_t reserved0;
  double du, dv, half_u, half_v;
  double sod, sdd;
  double start_plane;
} monte_mc_geom;

/*
 * Label-volume phantom, labels[nz][ny][nx] (uint8), voxel (ix,iy,iz)
 * covering x in [x0 + ix*dx, x0 + (ix+1)*dx) etc. (CBCT_real325im.cu:921:
 * x0 = y0 = z0 = -10 cm, d = 0.1 cm).  Label l is material label_material[l]
 * (an index into the XCOM tables, or -1 for air) at density
 * label_density[l] g/cm^3.  If clip_radius > 0, labels outside the cylinder
 * x^2+y^2 <= clip_radius^2, |z| <= clip_half_z read as air (:904).
 * `labels` follows the call's `mem`; the two label tables are host memory.
 */
typedef struct monte_mc_phantom {
  const uint8_t* labels;
  int32_t nx, ny, nz;
  int32_t n_labels;         /* <= 256 */
  double dx, dy, dz;
  double x0, y0, z0;
  double clip_radius, clip_half_z;
  const int32_t* label_material;
  const double* label_density;
} monte_mc_phantom;

/* XCOM mass coefficients [cm^2/g] per material, each [n_materials][201]
 * indexed by keV (row r of the reference CSV at index r,
 * monte_cpp/CBCT_real2.cpp:633-668).  Host memory. */
typedef struct monte_xcom {
  int32_t n_materials;      /* <= 8 */
  int32_t reserved0;
  const float* coherent;
  const float* incoherent;
  const float* photoelectric;
  const float* total;
} monte_xcom;

/* Source spectrum: discrete lines with relative weights (a single line is
 * monoenergetic; the reference forces 140 keV, CBCT_real325im.cu:491).
 * Host memory. */
typedef struct monte_spectrum {
  int32_t n_lines;          /* 1..512 */
  int32_t reserved0;
  const double* energy_kev;
  const double* weight;
} monte_spectrum;

/* What to simulate: `histories_per_pixel` histories aimed at every pixel
 * of [u_begin,u_end) x [v_begin,v_end) for every view of
 * [view_begin,view_end).  History k of (view, i, j) draws from the stream
 * ((view*nu + i)*nv + j)*histories_per_pixel + k of seed `seed`, job `job`,
 * so any split of the work reproduces the same tallies. */
typedef struct monte_mc_request {
  uint64_t seed;
  uint64_t histories_per_pixel;
  int32_t view_begin, view_end;
  int32_t u_begin, u_end, v_begin, v_end;
  int32_t kernel;           /* MONTE_MC_PLAIN / MONTE_MC_PERSISTENT */
  uint32_t job;
} monte_mc_request;

typedef struct monte_mc_stats {
  uint64_t histories;
  uint64_t woodcock_steps;
  uint64_t interactions;
  uint64_t primary_counts;  /* tallied */
  uint64_t scatter_counts;  /* tallied */
  uint64_t dropped;         /* histories stopped by a step or rejection cap */
  uint64_t rayleigh;        /* interactions by kind: coherent (no deflection), */
  uint64_t compton;         /* incoherent (Klein-Nishina), */
  uint64_t photoelectric;   /* photo-absorption */
  uint64_t majorant_legs;   /* moves of one macro-cell leg (MONTE_MC_LOCAL_MAJORANT) */
} monte_mc_stats;

/* Defaults equal to monte_cu/CBCT_real325im.cu: 360 views, 325x325 pixels
 * of 0.1 cm, SOD 160, SDD 220, start plane 10.1, 5 interactions,
 * MONTE_MC_STALE_SIN_PHI. */
void monte_mc_geom_reference325(monte_mc_geom* g);
/* Defaults equal to monte_cpp/CBCT_real2.cpp: 65x65 pixels of 0.5 cm, start
 * plane 6, 5 interactions, MONTE_MC_FIRST_COMPTON_Z | MONTE_MC_NO_RAYLEIGH_TALLY. */
void monte_mc_geom_reference_cpu(monte_mc_geom* g);

/* Parse one XCOM CSV (rows "coh,incoh,photo,total", UTF-8 BOM and CRLF
 * tolerated) into four [201] arrays indexed by keV.  Host only, no GPU. */
int monte_xcom_parse_csv(const char* text, size_t len, float* coherent, float* incoherent,
                         float* photoelectric, float* total);

/* The reference's source spectrum as lines (monte_cu/CBCT_real325.cu:
 * 349-389 reads the table, :479-486 samples it): cum[0..n_bins] is a
 * cumulative table over half-keV bins (250 bins in 125kv_al2mm.txt /
 * 125kv_al10mm.txt); a uniform u in (0, 1] selects the first bin d with
 * cum[d] <= u <= cum[d+1], energy (d + 1) * bin_kev, and falls back to
 * fallback_kev when no bin holds it (the reference's start_keV, 140).
 * Writes the n_bins + 1 lines (bin energies, then the fallback) with the
 * probability of each under that rule -- the reference's distribution
 * exactly, whatever the table (an all-zero table, what the reference's
 * reader leaves at :384, gives the fallback alone) -- for monte_spectrum.
 * energy_kev and weight hold n_bins + 1 doubles.  Host only, no GPU. */
int monte_spectrum_from_cumulative(const float* cum, int32_t n_bins, double bin_kev,
                                   double fallback_kev, double* energy_kev, double* weight,
                                   int32_t* n_lines);

/* Whitespace-separated numbers of a text table (the reference's fscanf
 * "%f" reads of 125kv_al*.txt, CBCT_real325.cu:363-386) into values;
 * *n_values = how many were read (at most max_values).  Host only. */
int monte_parse_numbers(const char* text, size_t len, float* values, int32_t max_values,
                        int32_t* n_values);

/* Draw the source energies of histories 0..n-1 of stream (seed, job) with
 * the Monte Carlo kernels' own sampler (the first draw of every history of
 * monte_mc_run, an alias table over the lines), into energies[n] (float
 * keV, following `mem`).  No counterpart in the reference: it shows the
 * sampled spectrum without running transport. */
int monte_mc_sample_energies(monte_ctx* ctx, const monte_spectrum* spec, uint64_t seed,
                             uint32_t job, uint64_t n, float* energies, int mem);

/* Run the Monte Carlo.  primary and scatter are int64 [n_views][nu][nv]
 * tallies that the call ADDS to (zero them first); they follow `mem`.
 * With MONTE_MEM_DEVICE the labels and both tallies must be memory the GPU
 * addresses directly (device, managed, or pinned host memory mapped at the
 * same address); anything else is rejected with MONTE_EINVAL before any
 * work.  stats may be NULL.  Replaces the projection launch of
 * monte_cu/CBCT_real325im.cu:235-248. */
int monte_mc_run(monte_ctx* ctx, const monte_mc_geom* g, const monte_mc_phantom* ph,
                 const monte_xcom* xcom, const monte_spectrum* spec, const monte_mc_request* run,
                 int64_t* primary, int64_t* scatter, monte_mc_stats* stats, int mem);

/* Limits of monte_mc_run_noalloc's static scratch. */
#define MONTE_NOALLOC_MAX_VIEWS  1024
#define MONTE_NOALLOC_MAX_PIXELS 1024

/* monte_mc_run for callers that cannot allocate device memory -- a service
 * that reserves all of the GPU's memory for its own pool, a framework whose
 * allocator must own every device allocation, a latency-critical loop where
 * a cudaMalloc (which can synchronize the device) is not acceptable.  It has
 * no counterpart in the reference.  It needs no context and allocates
 * nothing: the tables, the history counter and the statistics live in a
 * static device array of about 280 KB that every GPU loading the library
 * holds until exit.  Same semantics as monte_mc_run with the persistent or
 * plain kernel, on the current device and `cuda_stream` (NULL: the legacy
 * default stream); labels, primary and scatter must be device (or managed)
 * memory, else MONTE_EINVAL.  Requests with more than
 * MONTE_NOALLOC_MAX_VIEWS views or MONTE_NOALLOC_MAX_PIXELS pixels along an
 * axis are rejected (MONTE_EINVAL), and so is MONTE_MC_LOCAL_MAJORANT
 * (MONTE_EUNSUPPORTED: its per-phantom tables do not fit the array).  The
 * first call on a device looks up the array's address
 * (cudaGetSymbolAddress) and keeps it for the process's life: do not
 * cudaDeviceReset a device between calls.  The call cannot be captured into
 * a CUDA graph (its tables go up from host staging the next call reuses):
 * on a capturing stream it returns MONTE_EUNSUPPORTED and issues nothing.
 * All calls on a device share the array, which keeps the last call's
 * contents: calls whose work overlaps on the GPU race and must be
 * serialized; calls queued one after another on one stream are fine.  If
 * stats is not NULL the call waits for the stream.  Errors:
 * monte_last_error(NULL). */
int monte_mc_run_noalloc(const monte_mc_geom* g, const monte_mc_phantom* ph,
                         const monte_xcom* xcom, const monte_spectrum* spec,
                         const monte_mc_request* run, int64_t* primary, int64_t* scatter,
                         monte_mc_stats* stats, void* cuda_stream);

/* Reference post-processing (monte_cu/CBCT_real325im.cu:261-294): counts
 * clamped to [1, per]; map = -ln N + ln(per).  proj0/map0 from the primary
 * tally, proj5/map5 from primary + scatter; any output may be NULL.  All
 * arrays [n_views][nu][nv], following `mem`. */
int monte_mc_finalize(monte_ctx* ctx, int32_t n_views, int32_t nu, int32_t nv, uint64_t per,
                      const int64_t* primary, const int64_t* scatter, int32_t* proj0,
                      float* map0, int32_t* proj5, float* map5, int mem);

/* ======================================================================
 *  Batched scans (serving-style)
 * ====================================================================== */

/*
 * One simulated scan of a batch: the Monte Carlo of a phantom (the
 * projection launch plus post-processing of monte_cu/CBCT_real325im.cu:
 * 235-294), then the FDK reconstruction of its -log map
 * (recon/bp3d20.cpp:15-194), which reads the map as proj[view][u][v].  The
 * reference runs one phantom per program invocation; the batch has no
 * counterpart there.
 *
 * fdk.n_views, fdk.nu, fdk.nv must equal mc.n_views, mc.nu, mc.nv.  The
 * labels and every output are device pointers.  History streams are those of
 * monte_mc_run with request {seed, histories_per_pixel, all views and
 * pixels, job = the job's index in the batch}.
 */
typedef struct monte_batch_job {
  monte_mc_geom mc;
  monte_mc_phantom phantom;
  monte_spectrum spectrum;
  uint64_t seed;
  uint64_t histories_per_pixel;
  monte_fdk_geom fdk;
  int32_t recon_total;      /* 0: reconstruct map0 (primary only),
                               1: map5 (primary + scatter) */
  int32_t reserved0;
  int64_t* primary;         /* [n_views][nu][nv] tallies, zeroed by every run */
  int64_t* scatter;
  float* map;               /* [n_views][nu][nv] map the FDK reads; NULL: plan-owned */
  float* vol_xy;            /* [nz][ny][nx] reconstruction */
} monte_batch_job;

/* Batch execution forms. */
#define MONTE_BATCH_FUSED      0 /* one persistent Monte Carlo launch over the
                                    histories of all jobs, then per job finalize,
                                    split-BF16 tensor-core filter (FP32 where the
                                    detector does not fit it) and tiled
                                    backprojection, the jobs spread over four
                                    streams; all captured once in a CUDA graph */
#define MONTE_BATCH_SEQUENTIAL 1 /* per job, one after another: plain Monte
                                    Carlo kernel, finalize, FP32 filter, plain
                                    backprojection (no graph) */
/* monte_batch_create option bits. */
#define MONTE_BATCH_AUTOTUNE 0x1 /* time the leading tile shapes of the tiled
                                    backprojector on every distinct FDK
                                    geometry at creation (FUSED only); the
                                    full sweep is monte_fdk_autotune */

typedef struct monte_batch monte_batch;

/* Validate the jobs, build and upload every table, allocate the plan's
 * device memory and, for MONTE_BATCH_FUSED, capture the CUDA graph.  The
 * job array is copied; the buffers it points at must outlive the plan.
 * xcom is shared by all jobs.  At most 1024 jobs. */
int monte_batch_create(monte_ctx* ctx, const monte_xcom* xcom, const monte_batch_job* jobs,
                       int n_jobs, int mode, int options, monte_batch** out);
/* Queue one run of the whole batch on the context's stream (asynchronous). */
int monte_batch_run(monte_batch* b);
/* Statistics of the last run (waits for the context's stream). */
int monte_batch_stats(monte_batch* b, monte_mc_stats* stats);
/* Tile shape the backprojection of job j runs with (-1: plain kernel). */
int monte_batch_bp_variant(const monte_batch* b, int job);
int monte_batch_destroy(monte_batch* b);

/* ======================================================================
 *  Primary signal (differentiable mode)
 * ====================================================================== */

/* Voxel grid of an attenuation volume mu[nz][ny][nx] (1/cm), same
 * conventions as monte_mc_phantom. */
typedef struct monte_siddon_grid {
  int32_t nx, ny, nz, reserved0;
  double dx, dy, dz;
  double x0, y0, z0;
} monte_siddon_grid;

/* Expected primary signal of the Monte Carlo: for every pixel (i, j) of the
 * views [view_begin, view_end), the line integral L of mu along the
 * emission ray the Monte Carlo aims at that pixel
 * (monte_cu/CBCT_real325im.cu:476-512) by Siddon's exact voxel traversal,
 * and the transmission exp(-L) -- the expectation of the primary tally per
 * history (:567-590).  line / transmission are [n_views][nu][nv] (either may
 * be NULL); only the requested views are written. */
int monte_siddon_forward(monte_ctx* ctx, const monte_mc_geom* g, const monte_siddon_grid* grid,
                         const float* mu, int view_begin, int view_end, float* line,
                         float* transmission, int mem);
/* Adjoint of monte_siddon_forward: grad_mu[v] += sum over rays of
 * (grad_line + grad_transmission * d exp(-L)/dL) * (length of the ray in
 * voxel v).  The line integrals are recomputed, not read back.  Either
 * gradient may be NULL.  The per-voxel sums are int64 fixed point, with a
 * power-of-two scale chosen from the largest incoming gradient so that no
 * sum can overflow, so grad_mu is the same bit for bit in every run
 * whatever order the rays finish in; a non-finite incoming gradient makes
 * grad_mu NaN. */
int monte_siddon_backward(monte_ctx* ctx, const monte_mc_geom* g, const monte_siddon_grid* grid,
                          const float* mu, int view_begin, int view_end, const float* grad_line,
                          const float* grad_transmission, float* grad_mu, int mem);

#ifdef __cplusplus
}
#endif
#endif /* MONTE_H */
