// monte_fdk -- drop-in for the reference FDK programs recon/bp3d20.cpp and
// recon/bp3d20_325.cpp: reads the same projection file, writes the same three
// raw outputs (xy volume, zy volume, filtered map) under the same names,
// with the reconstruction running on the GPU through libmonte.
//
//   monte_fdk [--preset 65|325] [--in FILE] [--stem STEM] [--filter fp32|bf16x3]
//             [--bp plain|tiled] [--full]
//
// Defaults follow the reference: preset 65 reads mapg_0_20000h2oCa.raw and
// writes CBCTrecon\xy2mh20kyu2.raw, CBCTrecon\zy2mh20kyu2.raw,
// CBCTrecon\map2mh20kyu2.raw (recon/bp3d20.cpp:5-7,28,170-190; the names
// keep the reference's literal backslash).  Preset 325 reads
// mapg325_0_2tca.raw and writes the *ca0_2t files (recon/bp3d20_325.cpp).
// --full reconstructs the whole 256^3 grid instead of the reference's
// s in [125,130) slab.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "include/monte.h"

static int fail(const char* what, monte_ctx* ctx) {
  fprintf(stderr, "monte_fdk: %s: %s\n", what, monte_last_error(ctx));
  return 1;
}

int main(int argc, char** argv) {
  std::string preset = "65", in, stem, filter = "fp32", bp = "tiled";
  bool full = false;
  for (int i = 1; i < argc; i++) {
    std::string a = argv[i];
    auto next = [&]() -> std::string {
      if (i + 1 >= argc) {
        fprintf(stderr, "monte_fdk: %s needs a value\n", a.c_str());
        exit(2);
      }
      return argv[++i];
    };
    if (a == "--preset") preset = next();
    else if (a == "--in") in = next();
    else if (a == "--stem") stem = next();
    else if (a == "--filter") filter = next();
    else if (a == "--bp") bp = next();
    else if (a == "--full") full = true;
    else {
      fprintf(stderr, "usage: monte_fdk [--preset 65|325] [--in FILE] [--stem STEM] "
                      "[--filter fp32|bf16x3] [--bp plain|tiled] [--full]\n");
      return 2;
    }
  }
  monte_fdk_geom g;
  if (preset == "65") {
    monte_fdk_geom_reference65(&g);
    if (in.empty()) in = "mapg_0_20000h2oCa.raw";
    if (stem.empty()) stem = "2mh20kyu2";
  } else if (preset == "325") {
    monte_fdk_geom_reference325(&g);
    if (in.empty()) in = "mapg325_0_2tca.raw";
    if (stem.empty()) stem = "ca0_2t";
  } else {
    fprintf(stderr, "monte_fdk: unknown preset %s\n", preset.c_str());
    return 2;
  }
  if (full) {
    g.s_begin = 0;
    g.s_end = g.nx;
  }
  const size_t np = (size_t)g.n_views * g.nu * g.nv;
  const size_t nvol = (size_t)g.nx * g.ny * g.nz;
  std::vector<float> proj(np), filtered(np), xy(nvol), zy(nvol);
  FILE* f = fopen(in.c_str(), "rb");
  if (!f) {
    fprintf(stderr, "monte_fdk: failed to open %s\n", in.c_str());
    return 1;
  }
  size_t got = fread(proj.data(), sizeof(float), np, f);
  fclose(f);
  if (got != np) {
    fprintf(stderr, "monte_fdk: %s holds %zu floats, expected %zu\n", in.c_str(), got, np);
    return 1;
  }
  monte_ctx* ctx = nullptr;
  if (monte_ctx_create(&ctx, 0) != MONTE_OK) return fail("context", nullptr);
  int fm = filter == "bf16x3" ? MONTE_FILTER_BF16X3 : MONTE_FILTER_FP32;
  int bm = bp == "plain" ? MONTE_BP_PLAIN : MONTE_BP_TILED;
  if (monte_fdk(ctx, &g, proj.data(), filtered.data(), xy.data(), zy.data(), fm, bm,
                MONTE_MEM_HOST) != MONTE_OK)
    return fail("fdk", ctx);
  monte_ctx_destroy(ctx);
  struct Out {
    std::string name;
    const std::vector<float>* data;
  } outs[] = {{"CBCTrecon\\xy" + stem + ".raw", &xy},
              {"CBCTrecon\\zy" + stem + ".raw", &zy},
              {"CBCTrecon\\map" + stem + ".raw", &filtered}};
  for (auto& o : outs) {
    FILE* w = fopen(o.name.c_str(), "wb");
    if (!w || fwrite(o.data->data(), sizeof(float), o.data->size(), w) != o.data->size()) {
      fprintf(stderr, "monte_fdk: failed to write %s\n", o.name.c_str());
      if (w) fclose(w);
      return 1;
    }
    fclose(w);
  }
  printf("filtered\n");
  return 0;
}
