// monte_mc -- drop-in for the reference GPU Monte Carlo
// monte_cu/CBCT_real325im.cu: reads the 200^3 label volume (cyu8_2.raw,
// 0.1 cm voxels, x0 = y0 = z0 = -10 cm, labels 1 water / 2 Ca / >= 3 PMMA
// inside the r = 9 cm cylinder, :18,86-95,904-921), runs `per` histories
// aimed at every pixel of every view, and writes the reference's four raw
// files: proj325_teth0...raw / map325_teth0...raw (primary) and
// proj325_teth5...raw / map325_teth5...raw (primary + scatter), int32 counts
// clamped to [1, per] and float -ln N + ln per (:22-26,261-294).
//
//   monte_mc [--labels FILE] [--xcom FILE] [--ca FILE] [--pmma FILE] [--kev E]
//            [--per N] [--views N] [--kernel persistent|plain] [--seed S]
//            [--textbook]
//
// The XCOM tables are read from the CSV files of the reference tree
// (monte_cpp/xcom2.csv, monte_cpp/Ca.csv); the reference's own .txt copies and
// its PMMA table are not in its tree, so labels >= 3 need --pmma.
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "include/monte.h"

static bool read_file(const std::string& path, std::vector<char>* out) {
  FILE* f = fopen(path.c_str(), "rb");
  if (!f) return false;
  fseek(f, 0, SEEK_END);
  long n = ftell(f);
  fseek(f, 0, SEEK_SET);
  out->resize((size_t)n);
  size_t got = fread(out->data(), 1, (size_t)n, f);
  fclose(f);
  return got == (size_t)n;
}

template <typename T>
static bool write_file(const std::string& path, const std::vector<T>& v) {
  FILE* f = fopen(path.c_str(), "wb");
  if (!f) return false;
  bool ok = fwrite(v.data(), sizeof(T), v.size(), f) == v.size();
  fclose(f);
  return ok;
}

int main(int argc, char** argv) {
  std::string labels_path = "cyu8_2.raw", xcom = "xcom2.csv", ca = "Ca.csv", pmma;
  std::string kernel = "persistent";
  double kev = 140.0;
  uint64_t per = 10000, seed = 0;
  int views = 360;
  bool textbook = false;
  for (int i = 1; i < argc; i++) {
    std::string a = argv[i];
    auto next = [&]() -> std::string {
      if (i + 1 >= argc) {
        fprintf(stderr, "monte_mc: %s needs a value\n", a.c_str());
        exit(2);
      }
      return argv[++i];
    };
    if (a == "--labels") labels_path = next();
    else if (a == "--xcom") xcom = next();
    else if (a == "--ca") ca = next();
    else if (a == "--pmma") pmma = next();
    else if (a == "--kev") kev = atof(next().c_str());
    else if (a == "--per") per = strtoull(next().c_str(), nullptr, 10);
    else if (a == "--views") views = atoi(next().c_str());
    else if (a == "--kernel") kernel = next();
    else if (a == "--seed") seed = strtoull(next().c_str(), nullptr, 10);
    else if (a == "--textbook") textbook = true;
    else {
      fprintf(stderr, "usage: monte_mc [--labels FILE] [--xcom FILE] [--ca FILE] [--pmma FILE] "
                      "[--kev E] [--per N] [--views N] [--kernel persistent|plain] [--seed S] "
                      "[--textbook]\n");
      return 2;
    }
  }
  const int n = 200;
  std::vector<char> raw;
  if (!read_file(labels_path, &raw) || raw.size() < (size_t)n * n * n) {
    fprintf(stderr, "monte_mc: failed to read %s (200^3 uint8 expected)\n", labels_path.c_str());
    return 1;
  }
  std::vector<uint8_t> labels(raw.begin(), raw.begin() + (size_t)n * n * n);
  int max_label = 0;
  for (uint8_t l : labels) max_label = l > max_label ? l : max_label;
  int n_mat = pmma.empty() ? 2 : 3;
  if (max_label >= 3 && pmma.empty()) {
    fprintf(stderr, "monte_mc: labels >= 3 (PMMA) present; pass --pmma TABLE.csv\n");
    return 1;
  }
  std::vector<float> tab(4 * 3 * 201, 0.f);  // [field][material][201]
  const std::string paths[3] = {xcom, ca, pmma};
  for (int m = 0; m < n_mat; m++) {
    std::vector<char> txt;
    if (!read_file(paths[m], &txt)) {
      fprintf(stderr, "monte_mc: failed to read %s\n", paths[m].c_str());
      return 1;
    }
    if (monte_xcom_parse_csv(txt.data(), txt.size(), &tab[(0 * 3 + m) * 201],
                             &tab[(1 * 3 + m) * 201], &tab[(2 * 3 + m) * 201],
                             &tab[(3 * 3 + m) * 201]) != MONTE_OK) {
      fprintf(stderr, "monte_mc: %s is not an XCOM csv\n", paths[m].c_str());
      return 1;
    }
  }
  // labels: 0 air, 1 water 1.0, 2 Ca 1.55, 3.. PMMA 1.18 (CBCT_real325im.cu:437-439)
  int n_labels = max_label + 1 < 3 ? 3 : max_label + 1;
  std::vector<int32_t> mat(n_labels, 2);
  std::vector<double> rho(n_labels, 1.18);
  mat[0] = -1;
  rho[0] = 0.0;
  mat[1] = 0;
  rho[1] = 1.0;
  mat[2] = 1;
  rho[2] = 1.55;
  monte_mc_phantom ph;
  memset(&ph, 0, sizeof(ph));
  ph.labels = labels.data();
  ph.nx = ph.ny = ph.nz = n;
  ph.n_labels = n_labels;
  ph.dx = ph.dy = ph.dz = 0.1;
  ph.x0 = ph.y0 = ph.z0 = -10.0;
  ph.clip_radius = 9.0;
  ph.clip_half_z = 10.0;
  ph.label_material = mat.data();
  ph.label_density = rho.data();
  monte_xcom x;
  memset(&x, 0, sizeof(x));
  x.n_materials = n_mat;
  // regroup into [material][201] per field
  std::vector<float> coh(n_mat * 201), inc(n_mat * 201), pho(n_mat * 201), tot(n_mat * 201);
  for (int m = 0; m < n_mat; m++)
    for (int k = 0; k < 201; k++) {
      coh[m * 201 + k] = tab[(0 * 3 + m) * 201 + k];
      inc[m * 201 + k] = tab[(1 * 3 + m) * 201 + k];
      pho[m * 201 + k] = tab[(2 * 3 + m) * 201 + k];
      tot[m * 201 + k] = tab[(3 * 3 + m) * 201 + k];
    }
  x.coherent = coh.data();
  x.incoherent = inc.data();
  x.photoelectric = pho.data();
  x.total = tot.data();
  double w = 1.0;
  monte_spectrum sp;
  memset(&sp, 0, sizeof(sp));
  sp.n_lines = 1;
  sp.energy_kev = &kev;
  sp.weight = &w;
  monte_mc_geom g;
  monte_mc_geom_reference325(&g);
  g.n_views = views;
  if (textbook) g.flags = 0;
  monte_mc_request rq;
  memset(&rq, 0, sizeof(rq));
  rq.seed = seed;
  rq.histories_per_pixel = per;
  rq.view_end = views;
  rq.u_end = g.nu;
  rq.v_end = g.nv;
  rq.kernel = kernel == "plain" ? MONTE_MC_PLAIN : MONTE_MC_PERSISTENT;
  const size_t cells = (size_t)views * g.nu * g.nv;
  std::vector<int64_t> prim(cells, 0), scat(cells, 0);
  std::vector<int32_t> proj0(cells), proj5(cells);
  std::vector<float> map0(cells), map5(cells);
  monte_ctx* ctx = nullptr;
  if (monte_ctx_create(&ctx, 0) != MONTE_OK) {
    fprintf(stderr, "monte_mc: %s\n", monte_last_error(nullptr));
    return 1;
  }
  monte_mc_stats st;
  if (monte_mc_run(ctx, &g, &ph, &x, &sp, &rq, prim.data(), scat.data(), &st, MONTE_MEM_HOST) != MONTE_OK ||
      monte_mc_finalize(ctx, views, g.nu, g.nv, per, prim.data(), scat.data(), proj0.data(),
                        map0.data(), proj5.data(), map5.data(), MONTE_MEM_HOST) != MONTE_OK) {
    fprintf(stderr, "monte_mc: %s\n", monte_last_error(ctx));
    return 1;
  }
  monte_ctx_destroy(ctx);
  printf("histories %llu  woodcock steps %llu  primary %llu  scatter %llu\n",
         (unsigned long long)st.histories, (unsigned long long)st.woodcock_steps,
         (unsigned long long)st.primary_counts, (unsigned long long)st.scatter_counts);
  if (!write_file("proj325_teth0pmma8etim2.raw", proj0) ||
      !write_file("map325_teth0pmma8etim2.raw", map0) ||
      !write_file("proj325_teth5pmma8etim2.raw", proj5) ||
      !write_file("map325_teth5pmma8etim2.raw", map5)) {
    fprintf(stderr, "monte_mc: failed to write the outputs\n");
    return 1;
  }
  return 0;
}
