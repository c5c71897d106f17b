// fdk.cuh -- device-side description of one FDK problem and the kernel
// launchers shared by fdk_filter.cu, fdk_bp.cu and fdk_api.cu.
#pragma once

#include <cuda_runtime.h>
#include <cstdint>
#include <vector>

#include "../../include/monte.h"
#include "bp_footprints.h"

namespace monte {

// Per-view constants of the backprojector, computed on the host in double
// (recon/bp3d20.cpp:85-88,103-104,134-137,159) and rounded to float.
//
// The detector coordinates of voxel column (s, t) in this view follow from
// two affine functions of the voxel indices,
//   Vx = A + s B + t C   (distance from the source along the central ray)
//   W  = D + s E + t F   (K Vy with K = sdd / du, Vy across the central ray)
// as y = half_u / du - W / Vx and x(z) = half_v / dv - (sdd / dv) Z(z) / Vx.
// Each coefficient is split into an exact part (suffix h: a multiple of one
// power of two per view and function, chosen so that the h-sum is exact in
// float for every voxel of the grid) and a small remainder (suffix l).  The
// kernels thus evaluate Vx and W to ~1e-12 relative in a few FMAs, and the
// coordinates to ~1e-8 pixel, where float arithmetic on the rotated voxel
// position alone leaves ~1e-5 pixel (the reference works in double).
struct alignas(16) BpView {  // 80 bytes: five vector loads per view
  float ah, bh, ch, al;
  float bl, cl, dh, eh;
  float fh, dl, el, fl;
  float c, s;     // cos, sin of the view angle
  float tanb;     // tan() as the distance term evaluates it
  float rs;       // 1/sqrt(1+tanb^2)
  float factor;   // dbeta * scale * scale2
  float px, py;   // rotated source position
  float pad;
};

// The same per-view constants in double, for re-evaluating voxel-view pairs
// that sit on a discontinuity of the reference's operator (see
// bp_ref_voxel below).
struct BpViewD {
  double c, s, px, py, tanb;
};

// Geometry as the kernels use it (float), derived from monte_fdk_geom, plus
// the double originals used by bp_ref_voxel.
struct FdkDev {
  double x0d, y0d, z0d, dvoxd, sddd, Dd;
  double half_ud, half_vd, inv_dud, inv_dvd;
  int n_views, nu, nv, nx, ny, nz;
  int s_begin, s_end;
  int mask_r2;           // <=0: no mask
  int cs, ct, cz;        // mask centre
  int flags;
  float x0, y0, z0, dvox;
  float sdd, D, sod;
  float half_u, half_v;
  float inv_du, inv_dv;
  // low parts of 1/du, 1/dv and dvox/dv (value - float(value)): a float
  // reciprocal pitch alone is a ~6e-8 scale error of every detector
  // coordinate, ~1e-5 pixel at column 128
  float inv_du_lo, inv_dv_lo;
  float dvox_inv_dv, dvox_inv_dv_lo;
  float xmax, ymax;      // accepted detector coordinate ranges [0,xmax], [0,ymax]
  // float pairs (hi + lo) of the constants of the exact coordinate path
  // (BpView): yc = half_u / du, xc = half_v / dv, kv = sdd / dv,
  // kb = sdd * dvox / dv (dx/dz times Vx), and z0, dvox
  float yc_h, yc_l, xc_h, xc_l;
  float kv_h, kv_l, kb_h, kb_l;
  float z0_h, z0_l, dz_h, dz_l;
};

// (h - p) / pitch as (h - p) * (inv_hi + inv_lo), the product rounded once.
__host__ __device__ __forceinline__ float bp_scale(float t, float inv_hi, float inv_lo) {
  return fmaf(t, inv_hi, t * inv_lo);
}

FdkDev make_fdk_dev(const monte_fdk_geom& g);

// Host copies of the per-geometry tables (fdk_api.cu): view constants in
// float and double, cosine weights [u][v], taps 0.5*h, and the pre-split
// Toeplitz operand of the tensor-core filter (empty if that filter does not
// fit the geometry).
struct FdkHostTables {
  std::vector<BpView> views;
  std::vector<BpViewD> viewsd;
  std::vector<float> weights;
  std::vector<float> taps;
  std::vector<uint16_t> bsplit;
};
void build_fdk_tables(const monte_fdk_geom* g, FdkHostTables* t);
// Argument checks of the FDK entry points (sets the context's error text).
int fdk_validate(monte_ctx* ctx, const monte_fdk_geom* g, bool need_grid);
// Time tiled backprojector shapes that fit g (`reps` launches each on the
// context's stream, the first discarded) into scratch `dv` from filtered
// projections `df`; *best = fastest shape, -1 if none fits.  candidates:
// the shapes to time (NULL: all of them); padded: the padded copy of df
// (launch_fdk_bp_tiled) or NULL.
int fdk_tune_bp(monte_ctx* ctx, const monte_fdk_geom* g, const BpView* views,
                const BpViewD* viewsd, const float* df, float* dv, int* best,
                const int* candidates, int n_candidates, int reps,
                const float* padded = nullptr, BpFootprints* footprints = nullptr);
// Shapes that led on the reference-size workloads, for quick tuning.
extern const int kBpQuickCandidates[];
extern const int kBpQuickCandidatesN;

// Kernel launchers (return cudaGetLastError()).
cudaError_t launch_fdk_filter_fp32(const FdkDev& d, const float* proj, const float* weights,
                                   const float* taps_half, float* filtered, cudaStream_t st);
cudaError_t launch_fdk_filter_bf16x3(const FdkDev& d, const float* proj, const float* weights,
                                     const uint16_t* bsplit, float* filtered, int* status,
                                     int sm_count, cudaStream_t st);
// Size in bytes of the pre-split, pre-tiled B operand of the BF16x3 filter.
size_t bf16x3_bsplit_bytes(int nu);
// Fill `out` (host) with the pre-split Toeplitz operand for the BF16x3 filter.
void bf16x3_build_bsplit(int nu, const float* taps_half, uint16_t* out);
bool bf16x3_supported(const FdkDev& d);

cudaError_t launch_fdk_bp_plain(const FdkDev& d, const BpView* views, const BpViewD* viewsd,
                                const float* filtered, float* vol_xy, float* vol_zy,
                                cudaStream_t st);
// One part of a backprojection: views [k_begin, k_end) of the geometry,
// the per-voxel sums starting from acc_in ([z][y][x], the sums over the
// views before k_begin) or from zero when acc_in is null.  Every voxel
// accumulates its views in index order whatever the split, so the parts
// of a backprojection give bit for bit the values of a single launch.
struct BpPart {
  int k_begin, k_end;
  const float* acc_in;
  // set by launch_fdk_bp_tiled: the footprint table of the per-warp
  // shapes (BpFootprints), or null (each warp projects its block's
  // corners itself)
  const int* footprints = nullptr;
};

// Counters after the status word (ints kBpExactSlot.. of the context's
// status array, two uint64): voxel-view pairs the tiled backprojectors
// decided in double (bp_ref_voxel) and (column, view) pairs whose distance
// weight's sign was taken in double (bp_ts_negative).
constexpr int kBpExactSlot = 8;
// status: device int set to 1 if a bounded wait gave up (MONTE_ETIMEOUT);
// part: NULL for all views from zero; padded: NULL, or a copy of filtered
// with its rows padded to a multiple of 4 floats (fdk_bp_pad_rows), from
// which the tiles are loaded when nu is not a multiple of 4 (a TMA row
// stride must be a multiple of 16 bytes); the exact per-voxel path always
// reads `filtered`.
// footprints: the caller's table cache (see BpFootprints), or null.
cudaError_t launch_fdk_bp_tiled(const FdkDev& d, const BpView* views, const BpViewD* viewsd,
                                const float* filtered, float* vol_xy, float* vol_zy,
                                int variant, int* status, cudaStream_t st,
                                const BpPart* part = nullptr, const float* padded = nullptr,
                                BpFootprints* footprints = nullptr);
// Row pitch (floats) of the padded copy, and the copy itself, of views
// [k_begin, k_end) (k_end < 0: to the last view).
inline int fdk_bp_pad_pitch(int nu) { return (nu + 3) & ~3; }
cudaError_t launch_fdk_bp_pad_rows(const FdkDev& d, const float* filtered, float* padded,
                                   cudaStream_t st, int k_begin = 0, int k_end = -1);
// Adjoints (fdk_adjoint.cu): forward projector = transpose of the plain
// backprojector, into filtered-space layout [view][v][u] (vol_z: scratch of
// fdk_fp_scratch_bytes for the volume's z-major copy and its column
// occupancy map); adjoint of the weighting + filter, [view][v][u] ->
// [view][u][v].
cudaError_t launch_fdk_forward_project(const FdkDev& d, const BpView* views, const BpViewD* viewsd,
                                       const float* vol, float* vol_z, float* out,
                                       cudaStream_t st);
inline size_t fdk_fp_scratch_bytes(const monte_fdk_geom& g) {
  return (size_t)g.nx * g.ny * g.nz * sizeof(float) + (size_t)g.nx * g.ny;
}
cudaError_t launch_fdk_filter_adjoint(const FdkDev& d, const float* g, const float* weights,
                                      const float* taps_half, float* h, cudaStream_t st);
int fdk_bp_tiled_variants();
// padded: the caller provides the padded copy of the filtered projections
// (needed by the per-warp shapes when nu is not a multiple of 4)
bool fdk_bp_tiled_supported(const FdkDev& d, int variant, bool padded = false);
// The tile shape to run: `want` when it fits the geometry, else the first
// of a fixed list of robust shapes that does (the one-warp shapes with 48
// and 32 voxels per lane, then two-warp and shared-ring ones), else -1
// (the plain backprojector).  want < 0: no choice made (not autotuned).
int fdk_bp_pick(const FdkDev& d, int want, bool padded = false);

#ifdef __CUDACC__
// Shared by the plain and tiled kernels: bilinear read of filtered[view]
// at detector coordinates (x: v row, y: u column), with the reference's
// flat-array semantics for neighbours past the last row/column.
__device__ __forceinline__ float bp_fetch(const float* __restrict__ f, size_t total, size_t idx,
                                          bool ok) {
  return (ok && idx < total) ? __ldg(f + idx) : 0.f;
}

__device__ __forceinline__ float bp_bilinear_global(const FdkDev& d, const float* __restrict__ f,
                                                    int k, float x, float y) {
  const size_t total = (size_t)d.n_views * d.nu * d.nv;
  int xi = (int)x, yi = (int)y;
  float fx = x - (float)xi, fy = y - (float)yi;
  size_t i00 = (size_t)k * d.nu * d.nv + (size_t)xi * d.nu + yi;
  bool flat = (d.flags & MONTE_FDK_FLAT_EDGE) != 0;
  float f00 = bp_fetch(f, total, i00, flat || (xi < d.nv && yi < d.nu));
  float f10 = bp_fetch(f, total, i00 + d.nu, flat || (xi + 1 < d.nv && yi < d.nu));
  float f01 = bp_fetch(f, total, i00 + 1, flat || (xi < d.nv && yi + 1 < d.nu));
  float f11 = bp_fetch(f, total, i00 + d.nu + 1, flat || (xi + 1 < d.nv && yi + 1 < d.nu));
  float r0 = fmaf(fx, f10 - f00, f00);
  float r1 = fmaf(fx, f11 - f01, f01);
  return fmaf(fy, r1 - r0, r0);
}

// Bilinear read at double coordinates (the weights rounded to float).
__device__ __forceinline__ float bp_bilinear_global_d(const FdkDev& d, const float* __restrict__ f,
                                                      int k, double x, double y) {
  const size_t total = (size_t)d.n_views * d.nu * d.nv;
  int xi = (int)x, yi = (int)y;
  float fx = (float)(x - xi), fy = (float)(y - yi);
  size_t i00 = (size_t)k * d.nu * d.nv + (size_t)xi * d.nu + yi;
  bool flat = (d.flags & MONTE_FDK_FLAT_EDGE) != 0;
  float f00 = bp_fetch(f, total, i00, flat || (xi < d.nv && yi < d.nu));
  float f10 = bp_fetch(f, total, i00 + d.nu, flat || (xi + 1 < d.nv && yi < d.nu));
  float f01 = bp_fetch(f, total, i00 + 1, flat || (xi < d.nv && yi + 1 < d.nu));
  float f11 = bp_fetch(f, total, i00 + d.nu + 1, flat || (xi + 1 < d.nv && yi + 1 < d.nu));
  float r0 = fmaf(fx, f10 - f00, f00);
  float r1 = fmaf(fx, f11 - f01, f01);
  return fmaf(fy, r1 - r0, r0);
}

// One voxel-view pair evaluated in double exactly as recon/bp3d20.cpp:95-142
// does (same operations, same order, no contraction): whether the voxel is
// rejected (:116), its detector coordinates x, y (:123-124 /
// bp3d20_325.cpp:134-135) and the distance weight D^2/(D-d)^2 (:134-142,159).
// The reference's operator jumps where tmp_s changes sign (the weight, when
// tan() is evaluated as the reference does) and at the detector edges, so
// pairs the float path finds within a small margin of those places are
// decided here.  Returns false when rejected.
__device__ __forceinline__ bool bp_ref_voxel(const FdkDev& d, const BpViewD& v, int s, int t,
                                             int z, double* x, double* y, double* w) {
  double X = __dadd_rn(d.x0d, __dmul_rn((double)s, d.dvoxd));
  double Y = __dsub_rn(d.y0d, __dmul_rn((double)t, d.dvoxd));
  double Z = __dsub_rn(d.z0d, __dmul_rn((double)z, d.dvoxd));
  double p0 = __dsub_rn(X, v.px), p1 = __dsub_rn(Y, v.py), p2 = Z;
  double tmp = p0;
  p0 = __dadd_rn(__dmul_rn(p0, v.c), __dmul_rn(p1, v.s));
  p1 = __dadd_rn(-__dmul_rn(tmp, v.s), __dmul_rn(p1, v.c));
  double to = __ddiv_rn(d.sddd, p0);
  p1 = __dmul_rn(p1, to);
  p2 = __dmul_rn(p2, to);
  if (fabs(p1) > d.half_ud || fabs(p2) > d.half_vd) return false;
  *y = -__dsub_rn(__dmul_rn(p1, d.inv_dud), __dmul_rn(d.half_ud, d.inv_dud));
  *x = -__dsub_rn(__dmul_rn(p2, d.inv_dvd), __dmul_rn(d.half_vd, d.inv_dvd));
  double ts = __dsub_rn(__dmul_rn(X, v.c), __dmul_rn(Y, v.s));
  double tt = __dadd_rn(__dmul_rn(X, v.s), __dmul_rn(Y, v.c));
  double dd = fabs(__dadd_rn(-__dmul_rn(v.tanb, tt), ts)) /
              __dsqrt_rn(__dadd_rn(1.0, __dmul_rn(v.tanb, v.tanb)));
  if (ts < 0) dd = -dd;
  double den = __dsub_rn(d.Dd, dd);
  *w = __ddiv_rn(__dmul_rn(d.Dd, d.Dd), __dmul_rn(den, den));
  return true;
}

// Voxel (X, Y) in the frame of view v: Vx along the central ray from the
// source, Vy across it.  The reference forms (X - px) c + (Y - py) s and
// (Y - py) c - (X - px) s in double (recon/bp3d20.cpp:103-110); with the
// source at px = -sod c, py = -sod s these equal X c + Y s + sod and
// Y c - X s exactly.  Written so, the sod-sized source terms never cancel in
// float: the detector column keeps ~1e-6 pixel accuracy where the
// difference form loses ~1e-4 pixel at fine detector pitch.
__device__ __forceinline__ void bp_view_frame(const FdkDev& d, const BpView& v, float X, float Y,
                                              float* Vx, float* Vy) {
  *Vx = fmaf(X, v.c, Y * v.s) + d.sod;
  *Vy = fmaf(Y, v.c, -(X * v.s));
}

// ---- exact detector coordinates (float pairs) ---------------------------

// An unevaluated sum h + l of two floats.
struct Fpair {
  float h, l;
};

// 1/v: the hardware approximation refined by one Newton-Raphson step,
// r + r (1 - v r), within an ulp of the correctly rounded reciprocal (v is
// a normal number here: a source distance or a squared weight distance).
__device__ __forceinline__ float rcp_nr(float v) {
  float r;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(v));
  return fmaf(r, fmaf(-v, r, 1.0f), r);
}

// The pair arithmetic below relies on every product and sum being rounded
// on its own (the error terms recover exactly what that rounding lost), so
// it is written with the _rn intrinsics, which the compiler never fuses,
// whatever -fmad says for the file that includes it.

// a * b for pairs, to ~2^-46 relative (the l * l term dropped).
__device__ __forceinline__ Fpair bp_mul(Fpair a, Fpair b) {
  const float p = __fmul_rn(a.h, b.h);
  return {p, fmaf(a.h, b.l, fmaf(a.l, b.h, fmaf(a.h, b.h, -p)))};
}

// c - p for pairs with |c.h| >= |p.h| (Dekker's fast two-sum on the high
// parts: their difference's rounding error is recovered exactly), then
// normalised so that h is the sum rounded to float and |l| <= ulp(h) / 2.
// The low parts of products (bp_mul) carry the affine remainders, up to
// ~1e-4 of the value; without the normalisation, floor(h) could miss the
// coordinate's integer part by one near an integer.
__device__ __forceinline__ Fpair bp_sub(Fpair c, Fpair p) {
  const float h = __fsub_rn(c.h, p.h);
  const float l = __fadd_rn(__fsub_rn(__fsub_rn(c.h, h), p.h), __fsub_rn(c.l, p.l));
  const float s = __fadd_rn(h, l);
  return {s, __fsub_rn(l, __fsub_rn(s, h))};
}

// 1 / (vh + vl) for |vl| << |vh|: vh's reciprocal, its exact residual
// e = 1 - vh rh, and the series rh (1 + e - q + q^2) with q = vl rh.
__device__ __forceinline__ Fpair bp_recip(float vh, float vl) {
  const float rh = rcp_nr(vh);
  const float e = fmaf(-vh, rh, 1.0f);
  const float q = __fmul_rn(vl, rh);
  return {rh, __fmul_rn(rh, fmaf(q, q, __fsub_rn(e, q)))};
}

// (sdd / dv) Z(z) with Z(z) = z0 - z dvox, as a pair: the z term of every
// detector row coordinate, x(z) = half_v / dv - bp_zterm(z) / Vx.
__device__ __forceinline__ Fpair bp_zterm(const FdkDev& d, int z) {
  const float zf = (float)z;
  const float p = __fmul_rn(zf, d.dz_h);
  const float pe = fmaf(zf, d.dz_h, -p);  // z dz_h = p + pe exactly
  const float h = __fsub_rn(d.z0_h, p);   // two-sum of z0_h and -p
  const float bb = __fsub_rn(h, d.z0_h);
  const float e = __fadd_rn(__fsub_rn(d.z0_h, __fsub_rn(h, bb)), __fsub_rn(-p, bb));
  const Fpair Z = {h, __fadd_rn(e, __fsub_rn(__fsub_rn(d.z0_l, pe), __fmul_rn(zf, d.dz_l)))};
  return bp_mul({d.kv_h, d.kv_l}, Z);
}

// Per (column, view): r = 1 / Vx and the detector column coordinate
// y = half_u / du - W / Vx of voxel column (sf, tf), both as pairs, and
// q = W / Vx rounded (|q| > half_u / du is the reference's |u'| > half_u,
// recon/bp3d20.cpp:116).
__device__ __forceinline__ void bp_column_exact(const FdkDev& d, const BpView& v, float sf,
                                                float tf, Fpair* r, Fpair* y, float* q) {
  const float sx = fmaf(sf, v.bh, fmaf(tf, v.ch, v.ah));  // exact
  const float lx = fmaf(sf, v.bl, fmaf(tf, v.cl, v.al));
  const float sw = fmaf(sf, v.eh, fmaf(tf, v.fh, v.dh));  // exact
  const float lw = fmaf(sf, v.el, fmaf(tf, v.fl, v.dl));
  *r = bp_recip(sx, lx);
  const Fpair qq = bp_mul({sw, lw}, *r);
  *q = qq.h;
  *y = bp_sub({d.yc_h, d.yc_l}, qq);
}

// floor(v) for |v| < 2^22, as a float and as an int, without conversions:
// v + 1.5 * 2^23 rounded down lies in [2^23, 2^24), where floats are the
// integers, and its bits minus those of 1.5 * 2^23 are floor(v).
__device__ __forceinline__ float bp_floor(float v, int* vi) {
  const float t = __fadd_rd(v, 12582912.0f);
  *vi = (int)(__float_as_uint(t) - 0x4B400000u);
  return __fsub_rn(t, 12582912.0f);
}

// The part of bp_coef that depends only on the voxel column (X, Y) and the
// view: computed once per column by loops that walk a column along z.
struct BpColumn {
  Fpair r;         // 1 / Vx
  float q;         // W / Vx = half_u / du - y, rounded
  float y;         // detector column coordinate, rounded
  float ts;        // the signed in-plane term of the distance weight
  float w;         // D^2 / (D - d)^2
  float fy;        // column fraction (to ~1e-8)
  int yi;          // column index
  bool near;       // u' or y near a discontinuity of the operator
  bool out;        // rejected whatever z (|u'| > half_u or y outside [0, ymax])
};

// Whether the reference's tmp_s (recon/bp3d20.cpp:134) is negative, with
// its double arithmetic (the same operations as bp_ref_voxel).  The
// distance weight changes sign with tmp_s, and that sign is the only
// discontinuity of the weight; the float ts decides it when clear of 0,
// this where it is not.  The value of the weight is continuous there, so
// the float form stays exact enough: only the sign is taken from here.  A
// column on the rotation axis (even grids) has ts ~ 0 in every view.
// Out of line, with scalar arguments: inlined, the compiler evaluates the
// double operations speculatively for every voxel-view (FP64 is slow on
// this GPU), and a reference to the geometry would copy a by-value kernel
// parameter to local memory.
static __device__ __noinline__ bool bp_ts_negative(double x0d, double y0d, double dvoxd,
                                                   const BpViewD* v, int s, int t) {
  const double X = __dadd_rn(x0d, __dmul_rn((double)s, dvoxd));
  const double Y = __dsub_rn(y0d, __dmul_rn((double)t, dvoxd));
  return __dsub_rn(__dmul_rn(X, v->c), __dmul_rn(Y, v->s)) < 0.0;
}

__device__ __forceinline__ void bp_column(const FdkDev& d, const BpView& v, const BpViewD& vd,
                                          int s, int t, float X, float Y, BpColumn* c) {
  Fpair y;
  bp_column_exact(d, v, (float)s, (float)t, &c->r, &y, &c->q);
  c->y = y.h;
  c->ts = X * v.c - Y * v.s;
  c->near = fabsf(fabsf(c->q) - d.yc_h) < 1e-4f * d.yc_h || fabsf(c->y - d.ymax) < 1e-3f ||
            fabsf(c->y) < 1e-3f;
  c->out = fabsf(c->q) > d.yc_h || !(c->y >= 0.f && c->y <= d.ymax);
  float tt = X * v.s + Y * v.c;
  float dd = fabsf(c->ts - v.tanb * tt) * v.rs;
  if (fabsf(c->ts) < 1e-4f ? bp_ts_negative(d.x0d, d.y0d, d.dvoxd, &vd, s, t) : c->ts < 0.f)
    dd = -dd;
  float den = d.D - dd;
  c->w = (d.D * d.D) / (den * den);
  const float yf = bp_floor(y.h, &c->yi);
  c->fy = __fadd_rn(__fsub_rn(y.h, yf), y.l);
}

// Coefficients of one voxel-view pair of the backprojection operator:
// vol[s,t,z] += w * factor * bilinear(F_k; xi + fx, yi + fy).  Returns false
// when the pair contributes nothing (rejected by recon/bp3d20.cpp:116, or
// outside the interpolation guard of :152).  m = bp_zterm(d, z).  The plain
// backprojector and its adjoint (the forward projector) both use it
// (directly or as bp_column + bp_coef_z, the same operations), so the two
// are exact transposes of each other.  Pairs within a small margin of a
// discontinuity are decided in double (bp_ref_voxel).
__device__ __forceinline__ bool bp_coef_z(const FdkDev& d, const BpColumn& c, const BpViewD& vd,
                                          int s, int t, int z, Fpair m, int* xi, int* yi,
                                          float* fx, float* fy, float* w,
                                          bool* in_double = nullptr) {
  const Fpair p = bp_mul(m, c.r);  // Z sdd / (dv Vx) = half_v / dv - x
  const Fpair x = bp_sub({d.xc_h, d.xc_l}, p);
  const bool near = c.near || fabsf(fabsf(p.h) - d.xc_h) < 1e-4f * d.xc_h ||
                    fabsf(x.h - d.xmax) < 1e-3f || fabsf(x.h) < 1e-3f;
  if (!near) {
    if (c.out || fabsf(p.h) > d.xc_h || !(x.h >= 0.f && x.h <= d.xmax)) return false;
    *w = c.w;
    const float xf = bp_floor(x.h, xi);
    *fx = __fadd_rn(__fsub_rn(x.h, xf), x.l);
    *yi = c.yi;
    *fy = c.fy;
    return true;
  }
  double xd, yd, wd;
  if (in_double) *in_double = true;
  if (!bp_ref_voxel(d, vd, s, t, z, &xd, &yd, &wd)) return false;
  if (!(xd >= 0.0 && xd <= (double)d.nv && yd >= 0.0 && yd <= (double)d.nu)) return false;
  *w = (float)wd;
  *xi = (int)xd;
  *yi = (int)yd;
  *fx = (float)(xd - *xi);
  *fy = (float)(yd - *yi);
  return true;
}

// bp_column + bp_coef_z for one voxel (m = bp_zterm(d, z)).
__device__ __forceinline__ bool bp_coef(const FdkDev& d, const BpView& v, const BpViewD& vd, int s,
                                        int t, int z, float X, float Y, Fpair m, int* xi, int* yi,
                                        float* fx, float* fy, float* w,
                                        bool* in_double = nullptr) {
  BpColumn c;
  bp_column(d, v, vd, s, t, X, Y, &c);
  return bp_coef_z(d, c, vd, s, t, z, m, xi, yi, fx, fy, w, in_double);
}

// Bilinear read at integer corner (xi, yi) with fractions (fx, fy), with the
// reference's flat-array edge semantics (see bp_bilinear_global).
__device__ __forceinline__ float bp_bilinear_at(const FdkDev& d, const float* __restrict__ f, int k,
                                                int xi, int yi, float fx, float fy) {
  const size_t total = (size_t)d.n_views * d.nu * d.nv;
  size_t i00 = (size_t)k * d.nu * d.nv + (size_t)xi * d.nu + yi;
  bool flat = (d.flags & MONTE_FDK_FLAT_EDGE) != 0;
  float f00 = bp_fetch(f, total, i00, flat || (xi < d.nv && yi < d.nu));
  float f10 = bp_fetch(f, total, i00 + d.nu, flat || (xi + 1 < d.nv && yi < d.nu));
  float f01 = bp_fetch(f, total, i00 + 1, flat || (xi < d.nv && yi + 1 < d.nu));
  float f11 = bp_fetch(f, total, i00 + d.nu + 1, flat || (xi + 1 < d.nv && yi + 1 < d.nu));
  float r0 = fmaf(fx, f10 - f00, f00);
  float r1 = fmaf(fx, f11 - f01, f01);
  return fmaf(fy, r1 - r0, r0);
}

#endif

}  // namespace monte
