// mc_api.cu -- C-ABI entry points of the Monte Carlo path (include/monte.h).
//
// Reference host program: main() of monte_cu/CBCT_real325im.cu:83-297 --
// read the label volume and XCOM tables, copy them to the GPU, launch
// `projection`, copy the int32 tallies back, clamp and take -log, write raw
// files.  Here: monte_mc_run (tables + launch, int64 tallies) and
// monte_mc_finalize (the post-processing, on the GPU).
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <string>
#include <utility>
#include <vector>

#include "mc.cuh"
#include "mc_setup.h"
#include "monte_internal.h"

namespace monte {

namespace {

int check_mem(monte_ctx* ctx, int mem) {
  if (mem != MONTE_MEM_DEVICE && mem != MONTE_MEM_HOST)
    return set_error(ctx, MONTE_EINVAL, "bad mem %d", mem);
  return MONTE_OK;
}

}  // namespace

int mc_build_macro(monte_ctx* ctx, const monte_mc_phantom* ph, const monte_xcom* x,
                   bool labels_on_device, const mc_params& P, mc_local_tables* L,
                   std::vector<uint16_t>* cls, std::vector<uint8_t>* key) {
  mc_setup_local(ph, x, L);
  const size_t cells = (size_t)P.mgx * P.mgy * P.mgz;
  const size_t nlab = (size_t)ph->nx * ph->ny * ph->nz;
  if (key) {
    // the class grid depends on the grid, mu per label and the labels
    const int dims[7] = {P.mgx, P.mgy, P.mgz, P.mshift, ph->nx, ph->ny, ph->nz};
    key->resize(sizeof(dims) + sizeof(L->mu));
    memcpy(key->data(), dims, sizeof(dims));
    memcpy(key->data() + sizeof(dims), L->mu, sizeof(L->mu));
    if (labels_on_device && *key == ctx->mc_macro_key && ctx->mc_label_bytes == nlab) {
      // same grid and attenuation: the tables hold if the labels are those
      // they were built from, which the device checks against its copy (a
      // 4-byte answer, where the label sets would be 32 bytes per cell)
      MONTE_TRY(ensure_slot(ctx, kScratchAux2, sizeof(int), "label comparison flag"));
      int* dflag = (int*)ctx->scratch[kScratchAux2].ptr;
      MONTE_CUDA(ctx, cudaMemsetAsync(dflag, 0, sizeof(int), ctx->stream));
      cudaError_t e = launch_bytes_differ(ph->labels, (const uint8_t*)ctx->mc_label_copy.ptr, nlab,
                                          dflag, ctx->sm_count, ctx->stream);
      if (e != cudaSuccess) return cuda_fail(ctx, e, "label comparison");
      int differ = 1;
      MONTE_CUDA(ctx, cudaMemcpyAsync(&differ, dflag, sizeof(int), cudaMemcpyDeviceToHost,
                                      ctx->stream));
      MONTE_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
      if (!differ) return MONTE_OK;  // cls left empty: reuse the device copy
    }
  }
  std::vector<uint64_t> bits(cells * 4);
  if (labels_on_device) {
    MONTE_TRY(ensure_slot(ctx, kScratchAux3, cells * 4 * sizeof(uint64_t), "macro-cell label sets"));
    unsigned long long* db = (unsigned long long*)ctx->scratch[kScratchAux3].ptr;
    cudaError_t e = launch_mc_macro_bits(ph->labels, P, db, ctx->stream);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "macro-cell label sets");
    MONTE_CUDA(ctx, cudaMemcpyAsync(bits.data(), db, bits.size() * sizeof(uint64_t),
                                    cudaMemcpyDeviceToHost, ctx->stream));
    MONTE_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  } else {
    mc_macro_bits_host(ph, ph->labels, &P, bits.data());
    if (key) {
      // host labels: the cells' label sets complete the key
      const size_t k0 = key->size();
      key->resize(k0 + bits.size() * sizeof(uint64_t));
      memcpy(key->data() + k0, bits.data(), bits.size() * sizeof(uint64_t));
      if (*key == ctx->mc_macro_key) return MONTE_OK;  // cls left empty: reuse
    }
  }
  cls->assign(cells, 0);
  if (mc_macro_classes(&P, L, bits.data(), cls->data()) != MONTE_OK)
    return set_error(ctx, MONTE_ENOMEM, "out of host memory for the majorant classes");
  return MONTE_OK;
}

}  // namespace monte

using namespace monte;

extern "C" {

void monte_mc_geom_reference325(monte_mc_geom* g) {
  if (!g) return;
  memset(g, 0, sizeof(*g));
  g->n_views = 360;            // CBCT_real325im.cu:15
  g->nu = g->nv = 325;         // :9-10
  g->max_interactions = 5;     // :7
  g->flags = MONTE_MC_STALE_SIN_PHI;
  g->du = g->dv = 0.1;         // :459
  g->half_u = g->half_v = 16.25;
  g->sod = 160;
  g->sdd = 220;
  g->start_plane = 10.1;       // :460
}

void monte_mc_geom_reference_cpu(monte_mc_geom* g) {
  if (!g) return;
  memset(g, 0, sizeof(*g));
  g->n_views = 360;            // CBCT_real2.cpp:169 (only view 0 is run)
  g->nu = g->nv = 65;          // :60
  g->max_interactions = 5;     // :9
  g->flags = MONTE_MC_FIRST_COMPTON_Z | MONTE_MC_NO_RAYLEIGH_TALLY;
  g->du = g->dv = 0.5;         // :210
  g->half_u = g->half_v = 16.25;
  g->sod = 160;
  g->sdd = 220;
  g->start_plane = 6;          // :254
}

int monte_xcom_parse_csv(const char* text, size_t len, float* coherent, float* incoherent,
                         float* photoelectric, float* total) {
  if (!text || !coherent || !incoherent || !photoelectric || !total) return MONTE_EINVAL;
  std::string s(text, len);
  size_t pos = 0;
  if (s.size() >= 3 && (unsigned char)s[0] == 0xEF && (unsigned char)s[1] == 0xBB &&
      (unsigned char)s[2] == 0xBF)
    pos = 3;  // UTF-8 BOM (CBCT_real2.cpp:663 works around it with a literal)
  for (int k = 0; k < MC_NBINS; k++) coherent[k] = incoherent[k] = photoelectric[k] = total[k] = 0;
  int row = 0;
  while (pos < s.size() && row < MC_NBINS - 1) {
    size_t eol = s.find('\n', pos);
    if (eol == std::string::npos) eol = s.size();
    std::string line = s.substr(pos, eol - pos);
    pos = eol + 1;
    if (!line.empty() && line.back() == '\r') line.pop_back();
    bool blank = true;
    for (char c : line)
      if (c != ' ' && c != '\t') blank = false;
    if (blank) continue;
    float v[4];
    const char* p = line.c_str();
    for (int i = 0; i < 4; i++) {
      char* end = nullptr;
      v[i] = strtof(p, &end);
      if (end == p) return MONTE_EINVAL;
      p = end;
      while (*p == ' ' || *p == '\t') p++;
      if (i < 3) {
        if (*p != ',') return MONTE_EINVAL;
        p++;
      }
    }
    row++;  // row r (1-based) -> index r = keV
    coherent[row] = v[0];
    incoherent[row] = v[1];
    photoelectric[row] = v[2];
    total[row] = v[3];
  }
  if (row == 0) return MONTE_EINVAL;
  coherent[0] = coherent[1];
  incoherent[0] = incoherent[1];
  photoelectric[0] = photoelectric[1];
  total[0] = total[1];
  for (int k = row + 1; k < MC_NBINS; k++) {  // short tables: hold the last row
    coherent[k] = coherent[row];
    incoherent[k] = incoherent[row];
    photoelectric[k] = photoelectric[row];
    total[k] = total[row];
  }
  return MONTE_OK;
}

namespace {
// Whether the GPU can address p directly: device or managed memory, or
// pinned host memory mapped at the same address.  Pageable host memory
// (cudaMemoryTypeUnregistered) would fault the kernel.
bool gpu_addressable(const void* p) {
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged ||
         (a.type == cudaMemoryTypeHost && a.devicePointer == p);
}
}  // namespace

int monte_mc_run(monte_ctx* ctx, const monte_mc_geom* g, const monte_mc_phantom* ph,
                 const monte_xcom* xcom, const monte_spectrum* spec, const monte_mc_request* run,
                 int64_t* primary, int64_t* scatter, monte_mc_stats* stats, int mem) {
  if (!ctx) return MONTE_EINVAL;
  if (!g || !ph || !xcom || !spec || !run || !primary || !scatter || !ph->labels)
    return set_error(ctx, MONTE_EINVAL, "null argument");
  MONTE_TRY(check_mem(ctx, mem));
  if (mem == MONTE_MEM_DEVICE &&
      !(gpu_addressable(ph->labels) && gpu_addressable(primary) && gpu_addressable(scatter)))
    return set_error(ctx, MONTE_EINVAL,
                     "MONTE_MEM_DEVICE: labels, primary and scatter must be device memory");
  mc_params P;
  const char* why = "";
  if (mc_setup_params(g, ph, run, &P, &why) != MONTE_OK) return set_error(ctx, MONTE_EINVAL, "%s", why);
  std::vector<mc_tables> T(1);
  if (mc_setup_tables(ph, xcom, spec, T.data(), &why) != MONTE_OK)
    return set_error(ctx, MONTE_EINVAL, "%s", why);
  const unsigned long long npix =
      (unsigned long long)(run->u_end - run->u_begin) * (unsigned long long)(run->v_end - run->v_begin);
  const unsigned long long nview = (unsigned long long)(run->view_end - run->view_begin);
  unsigned long long total = 0;
  if (npix && nview && run->histories_per_pixel) {
    if (npix * nview > (1ull << 62) / run->histories_per_pixel)
      return set_error(ctx, MONTE_EOVERFLOW, "too many histories");
    total = npix * nview * run->histories_per_pixel;
  }
  size_t nlab = (size_t)ph->nx * ph->ny * ph->nz;
  size_t ncell = (size_t)g->n_views * g->nu * g->nv;
  std::vector<mc_view> V(g->n_views);
  std::vector<mc_pixel> U(g->nu), W(g->nv);
  mc_setup_views(g, V.data());
  mc_setup_pixels(g, U.data(), W.data());
  MONTE_TRY(enter(ctx));
  const bool local = (P.flags & MC_F_LOCAL_MAJORANT) != 0;
  if (local) {
    // the tables and class grid of the last call are reused when they were
    // built from the same phantom contents and tables
    std::vector<uint16_t> cls;
    std::vector<mc_local_tables> Lt(1);
    std::vector<uint8_t> key;
    MONTE_TRY(mc_build_macro(ctx, ph, xcom, mem == MONTE_MEM_DEVICE, P, Lt.data(), &cls, &key));
    if (!cls.empty()) {
      ctx->mc_macro_key.clear();
      MONTE_TRY(ensure(ctx, ctx->mc_mclass, cls.size() * 2 + sizeof(mc_local_tables),
                       "local majorant tables"));
      MONTE_CUDA(ctx, cudaMemcpyAsync(ctx->mc_mclass.ptr, Lt.data(), sizeof(mc_local_tables),
                                      cudaMemcpyHostToDevice, ctx->stream));
      MONTE_CUDA(ctx, cudaMemcpyAsync((char*)ctx->mc_mclass.ptr + sizeof(mc_local_tables),
                                      cls.data(), cls.size() * 2, cudaMemcpyHostToDevice,
                                      ctx->stream));
      ctx->mc_label_bytes = 0;
      if (mem == MONTE_MEM_DEVICE) {
        // the labels these tables were built from, for the next call's check
        MONTE_TRY(ensure(ctx, ctx->mc_label_copy, nlab, "label copy"));
        MONTE_CUDA(ctx, cudaMemcpyAsync(ctx->mc_label_copy.ptr, ph->labels, nlab,
                                        cudaMemcpyDefault, ctx->stream));
        ctx->mc_label_bytes = nlab;
      }
      ctx->mc_macro_key.swap(key);
    }
  }
  MONTE_TRY(ensure(ctx, ctx->mc_tables, sizeof(mc_tables), "MC tables"));
  MONTE_TRY(ensure(ctx, ctx->mc_views, V.size() * sizeof(mc_view), "MC view table"));
  MONTE_TRY(ensure(ctx, ctx->mc_pixels, (U.size() + W.size()) * sizeof(mc_pixel), "MC pixel table"));
  MONTE_TRY(ensure_slot(ctx, kScratchStats, 16 * sizeof(unsigned long long), "MC counters"));
  MONTE_CUDA(ctx, cudaMemcpyAsync(ctx->mc_tables.ptr, T.data(), sizeof(mc_tables),
                                  cudaMemcpyHostToDevice, ctx->stream));
  MONTE_CUDA(ctx, cudaMemcpyAsync(ctx->mc_views.ptr, V.data(), V.size() * sizeof(mc_view),
                                  cudaMemcpyHostToDevice, ctx->stream));
  mc_pixel* dpix = (mc_pixel*)ctx->mc_pixels.ptr;
  MONTE_CUDA(ctx, cudaMemcpyAsync(dpix, U.data(), U.size() * sizeof(mc_pixel),
                                  cudaMemcpyHostToDevice, ctx->stream));
  MONTE_CUDA(ctx, cudaMemcpyAsync(dpix + U.size(), W.data(), W.size() * sizeof(mc_pixel),
                                  cudaMemcpyHostToDevice, ctx->stream));
  unsigned long long* dstat = (unsigned long long*)ctx->scratch[kScratchStats].ptr;
  MONTE_CUDA(ctx, cudaMemsetAsync(dstat, 0, 16 * sizeof(unsigned long long), ctx->stream));
  const uint8_t* dlab = ph->labels;
  int64_t *dprim = primary, *dscat = scatter;
  if (mem == MONTE_MEM_HOST) {
    MONTE_TRY(ensure_slot(ctx, kScratchLabels, nlab, "label staging"));
    MONTE_TRY(ensure_slot(ctx, kScratchMcPrimary, ncell * 8, "tally staging"));
    MONTE_TRY(ensure_slot(ctx, kScratchMcScatter, ncell * 8, "tally staging"));
    MONTE_CUDA(ctx, cudaMemcpyAsync(ctx->scratch[kScratchLabels].ptr, ph->labels, nlab,
                                    cudaMemcpyHostToDevice, ctx->stream));
    MONTE_CUDA(ctx, cudaMemcpyAsync(ctx->scratch[kScratchMcPrimary].ptr, primary, ncell * 8,
                                    cudaMemcpyHostToDevice, ctx->stream));
    MONTE_CUDA(ctx, cudaMemcpyAsync(ctx->scratch[kScratchMcScatter].ptr, scatter, ncell * 8,
                                    cudaMemcpyHostToDevice, ctx->stream));
    dlab = (const uint8_t*)ctx->scratch[kScratchLabels].ptr;
    dprim = (int64_t*)ctx->scratch[kScratchMcPrimary].ptr;
    dscat = (int64_t*)ctx->scratch[kScratchMcScatter].ptr;
  }
  McDev d;
  memset(&d, 0, sizeof(d));
  d.P = P;
  d.T = (const mc_tables*)ctx->mc_tables.ptr;
  d.V = (const mc_view*)ctx->mc_views.ptr;
  d.U = dpix;
  d.W = dpix + U.size();
  d.labels = dlab;
  d.L = local ? (const mc_local_tables*)ctx->mc_mclass.ptr : nullptr;
  d.mclass = local ? (const uint16_t*)((const char*)ctx->mc_mclass.ptr + sizeof(mc_local_tables))
                   : nullptr;
  d.prim = (unsigned long long*)dprim;
  d.scat = (unsigned long long*)dscat;
  d.stats = dstat;
  d.counter = dstat + 12;
  d.total = total;
  if (total) {
    cudaError_t e = launch_mc(d, run->kernel, ctx->sm_count, ctx->stream);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "Monte Carlo launch");
  }
  if (mem == MONTE_MEM_HOST) {
    MONTE_CUDA(ctx, cudaMemcpyAsync(primary, dprim, ncell * 8, cudaMemcpyDeviceToHost, ctx->stream));
    MONTE_CUDA(ctx, cudaMemcpyAsync(scatter, dscat, ncell * 8, cudaMemcpyDeviceToHost, ctx->stream));
  }
  if (stats || mem == MONTE_MEM_HOST) {
    unsigned long long h[kMcStats];
    MONTE_CUDA(ctx, cudaMemcpyAsync(h, dstat, sizeof(h), cudaMemcpyDeviceToHost, ctx->stream));
    MONTE_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    if (stats) mc_stats_from(h, stats);
  }
  return MONTE_OK;
}

int monte_spectrum_from_cumulative(const float* cum, int32_t n_bins, double bin_kev,
                                   double fallback_kev, double* energy_kev, double* weight,
                                   int32_t* n_lines) {
  if (!cum || !energy_kev || !weight || !n_lines || n_bins <= 0 || n_bins + 1 > MC_MAX_LINES ||
      !(bin_kev > 0) || !(fallback_kev > 0))
    return MONTE_EINVAL;
  // u is uniform on (0, 1]; bin d takes the part of [cum[d], cum[d+1]]
  // inside (0, 1] that no earlier bin took (the reference's loop breaks at
  // the first match).  `taken` is the union of the earlier intervals as
  // disjoint sorted pieces.
  std::vector<std::pair<double, double>> taken;
  double total = 0.0;
  for (int d = 0; d < n_bins; d++) {
    double a = std::fmax((double)cum[d], 0.0), b = std::fmin((double)cum[d + 1], 1.0);
    double w = 0.0;
    if (b > a) {
      w = b - a;
      for (const auto& t : taken) w -= std::fmax(0.0, std::fmin(b, t.second) - std::fmax(a, t.first));
      std::vector<std::pair<double, double>> merged;
      bool placed = false;
      for (const auto& t : taken) {
        if (t.second < a || t.first > b) {
          if (!placed && t.first > b) {
            merged.push_back({a, b});
            placed = true;
          }
          merged.push_back(t);
        } else {
          a = std::fmin(a, t.first);
          b = std::fmax(b, t.second);
        }
      }
      if (!placed) merged.push_back({a, b});
      taken.swap(merged);
    }
    energy_kev[d] = (d + 1) * bin_kev;
    weight[d] = std::fmax(w, 0.0);
    total += weight[d];
  }
  energy_kev[n_bins] = fallback_kev;
  weight[n_bins] = std::fmax(1.0 - total, 0.0);
  *n_lines = n_bins + 1;
  return MONTE_OK;
}

int monte_parse_numbers(const char* text, size_t len, float* values, int32_t max_values,
                        int32_t* n_values) {
  if (!text || !values || !n_values || max_values < 0) return MONTE_EINVAL;
  std::string buf(text, len);
  const char* p = buf.c_str();
  int n = 0;
  while (n < max_values) {
    char* end = nullptr;
    const float v = strtof(p, &end);
    if (end == p) break;
    values[n++] = v;
    p = end;
  }
  *n_values = n;
  return MONTE_OK;
}

int monte_mc_sample_energies(monte_ctx* ctx, const monte_spectrum* spec, uint64_t seed,
                             uint32_t job, uint64_t n, float* energies, int mem) {
  if (!ctx) return MONTE_EINVAL;
  if (!spec || (!energies && n)) return set_error(ctx, MONTE_EINVAL, "null argument");
  MONTE_TRY(check_mem(ctx, mem));
  std::vector<mc_tables> T(1);
  memset(T.data(), 0, sizeof(mc_tables));
  const char* why = "";
  if (mc_setup_spectrum(spec, T.data(), &why) != MONTE_OK)
    return set_error(ctx, MONTE_EINVAL, "%s", why);
  if (n == 0) return MONTE_OK;
  if (n > ((uint64_t)1 << 40)) return set_error(ctx, MONTE_EOVERFLOW, "too many samples");
  MONTE_TRY(enter(ctx));
  MONTE_TRY(ensure(ctx, ctx->mc_tables, sizeof(mc_tables), "MC tables"));
  MONTE_CUDA(ctx, cudaMemcpyAsync(ctx->mc_tables.ptr, T.data(), sizeof(mc_tables),
                                  cudaMemcpyHostToDevice, ctx->stream));
  float* dout = energies;
  if (mem == MONTE_MEM_HOST) {
    MONTE_TRY(ensure_slot(ctx, kScratchAux0, n * sizeof(float), "energy staging"));
    dout = (float*)ctx->scratch[kScratchAux0].ptr;
  }
  monte_philox_keys keys;
  monte_philox_schedule(seed, &keys);
  cudaError_t e = launch_mc_energies((const mc_tables*)ctx->mc_tables.ptr, seed, keys, job, n,
                                     dout, ctx->sm_count, ctx->stream);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "energy sampling launch");
  if (mem == MONTE_MEM_HOST)
    MONTE_CUDA(ctx, cudaMemcpyAsync(energies, dout, n * sizeof(float), cudaMemcpyDeviceToHost,
                                    ctx->stream));
  // the host table dies at return
  MONTE_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return MONTE_OK;
}

int monte_mc_finalize(monte_ctx* ctx, int32_t n_views, int32_t nu, int32_t nv, uint64_t per,
                      const int64_t* primary, const int64_t* scatter, int32_t* proj0,
                      float* map0, int32_t* proj5, float* map5, int mem) {
  if (!ctx) return MONTE_EINVAL;
  MONTE_TRY(check_mem(ctx, mem));
  if (n_views <= 0 || nu <= 0 || nv <= 0 || per == 0 || per > (uint64_t)INT32_MAX)
    return set_error(ctx, MONTE_EINVAL, "bad finalize sizes");
  if (!primary) return set_error(ctx, MONTE_EINVAL, "null primary tally");
  if ((proj5 || map5) && !scatter)
    return set_error(ctx, MONTE_EINVAL, "proj5/map5 need the scatter tally");
  MONTE_TRY(enter(ctx));
  const size_t n = (size_t)n_views * nu * nv;
  // -log(N) + log(float(per)): the reference's log(float) overload
  // (CBCT_real325im.cu:284) rounds ln(per) to float.
  const double log_per = (double)(float)std::log((double)per);
  if (mem == MONTE_MEM_DEVICE) {
    cudaError_t e = launch_mc_finalize(n, per, log_per, (const long long*)primary,
                                       (const long long*)scatter, proj0, map0, proj5, map5,
                                       ctx->stream);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "finalize launch");
    return MONTE_OK;
  }
  MONTE_TRY(ensure_slot(ctx, kScratchMcPrimary, n * 8, "tally staging"));
  MONTE_TRY(ensure_slot(ctx, kScratchMcScatter, n * 8, "tally staging"));
  MONTE_TRY(ensure_slot(ctx, kScratchAux0, n * 4, "finalize staging"));
  MONTE_TRY(ensure_slot(ctx, kScratchAux1, n * 4, "finalize staging"));
  MONTE_TRY(ensure_slot(ctx, kScratchAux2, n * 4, "finalize staging"));
  MONTE_TRY(ensure_slot(ctx, kScratchAux3, n * 4, "finalize staging"));
  long long* dp = (long long*)ctx->scratch[kScratchMcPrimary].ptr;
  long long* ds = scatter ? (long long*)ctx->scratch[kScratchMcScatter].ptr : nullptr;
  int* d0 = (int*)ctx->scratch[kScratchAux0].ptr;
  float* m0 = (float*)ctx->scratch[kScratchAux1].ptr;
  int* d5 = (int*)ctx->scratch[kScratchAux2].ptr;
  float* m5 = (float*)ctx->scratch[kScratchAux3].ptr;
  MONTE_CUDA(ctx, cudaMemcpyAsync(dp, primary, n * 8, cudaMemcpyHostToDevice, ctx->stream));
  if (ds) MONTE_CUDA(ctx, cudaMemcpyAsync(ds, scatter, n * 8, cudaMemcpyHostToDevice, ctx->stream));
  cudaError_t e = launch_mc_finalize(n, per, log_per, dp, ds, proj0 ? d0 : nullptr,
                                     map0 ? m0 : nullptr, proj5 ? d5 : nullptr,
                                     map5 ? m5 : nullptr, ctx->stream);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "finalize launch");
  if (proj0) MONTE_CUDA(ctx, cudaMemcpyAsync(proj0, d0, n * 4, cudaMemcpyDeviceToHost, ctx->stream));
  if (map0) MONTE_CUDA(ctx, cudaMemcpyAsync(map0, m0, n * 4, cudaMemcpyDeviceToHost, ctx->stream));
  if (proj5) MONTE_CUDA(ctx, cudaMemcpyAsync(proj5, d5, n * 4, cudaMemcpyDeviceToHost, ctx->stream));
  if (map5) MONTE_CUDA(ctx, cudaMemcpyAsync(map5, m5, n * 4, cudaMemcpyDeviceToHost, ctx->stream));
  MONTE_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return MONTE_OK;
}

}  // extern "C"
