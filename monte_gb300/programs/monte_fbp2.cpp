// monte_fbp2 -- drop-in for the reference's 2-D fan-beam FBP program
// recon/fbp2.cpp: reads the same projection file (360 views x 65 elements,
// float), writes the same raw outputs under the same names (filtered
// projections and the 256x256 image), with the reconstruction running on the
// GPU through libmonte.
//
//   monte_fbp2 [--in FILE] [--image FILE] [--filtered FILE]
//
// Defaults follow the reference (recon/fbp2.cpp:5-7,29,153-165):
// map5_20_2e5.raw in, projection_test\outproj2e5.raw and
// projection_test\testxyo2e5.raw out (the names keep the reference's
// literal backslash).
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

#include "include/monte.h"

static int fail(const char* what, monte_ctx* ctx) {
  fprintf(stderr, "monte_fbp2: %s: %s\n", what, monte_last_error(ctx));
  return 1;
}

int main(int argc, char** argv) {
  std::string in = "map5_20_2e5.raw", image_name = "projection_test\\testxyo2e5.raw",
              filt_name = "projection_test\\outproj2e5.raw";
  for (int i = 1; i < argc; i++) {
    std::string a = argv[i];
    if (i + 1 >= argc) {
      fprintf(stderr, "usage: monte_fbp2 [--in FILE] [--image FILE] [--filtered FILE]\n");
      return 2;
    }
    if (a == "--in") in = argv[++i];
    else if (a == "--image") image_name = argv[++i];
    else if (a == "--filtered") filt_name = argv[++i];
    else {
      fprintf(stderr, "usage: monte_fbp2 [--in FILE] [--image FILE] [--filtered FILE]\n");
      return 2;
    }
  }
  monte_fbp2_geom g;
  monte_fbp2_geom_reference(&g);
  const size_t np = (size_t)g.n_views * g.n_det, ni = (size_t)g.nx * g.ny;
  std::vector<float> proj(np), filtered(np), image(ni);
  FILE* f = fopen(in.c_str(), "rb");
  if (!f) {
    fprintf(stderr, "monte_fbp2: failed to open %s\n", in.c_str());
    return 1;
  }
  size_t got = fread(proj.data(), sizeof(float), np, f);
  fclose(f);
  if (got != np) {
    fprintf(stderr, "monte_fbp2: %s holds %zu floats, expected %zu\n", in.c_str(), got, np);
    return 1;
  }
  monte_ctx* ctx = nullptr;
  if (monte_ctx_create(&ctx, 0) != MONTE_OK) return fail("context", nullptr);
  if (monte_fbp2(ctx, &g, proj.data(), filtered.data(), image.data(), MONTE_MEM_HOST) != MONTE_OK)
    return fail("fbp2", ctx);
  monte_ctx_destroy(ctx);
  struct Out {
    std::string name;
    const std::vector<float>* data;
  } outs[] = {{filt_name, &filtered}, {image_name, &image}};
  for (auto& o : outs) {
    FILE* w = fopen(o.name.c_str(), "wb");
    if (!w || fwrite(o.data->data(), sizeof(float), o.data->size(), w) != o.data->size()) {
      fprintf(stderr, "monte_fbp2: failed to write %s\n", o.name.c_str());
      if (w) fclose(w);
      return 1;
    }
    fclose(w);
  }
  printf("filtered\n");
  return 0;
}
