// bp_footprints.h -- the footprint table cache of the per-warp tiled
// backprojector shapes, owned by a context and filled by
// launch_fdk_bp_tiled (fdk_bp_tiled.cu).
#pragma once

#include <cstddef>
#include <cstdint>
#include <vector>

namespace monte {

// Footprints of the per-warp shapes' blocks, one int per (block, view):
// the tile origin and interior flag each warp would otherwise compute from
// its block's corners every four views.  launch_fdk_bp_tiled fills it for
// the geometry and shape it runs and rebuilds it when they change.  Tables
// above kBpFootprintMaxBytes are not built (the warps project their
// corners instead).
struct BpFootprints {
  int* ptr = nullptr;
  size_t bytes = 0;
  std::vector<uint8_t> key;  // the FdkDev and shape the contents are for
};
constexpr size_t kBpFootprintMaxBytes = size_t(256) << 20;
// Frees the table (the caller makes sure no queued work still reads it).
void fdk_bp_footprints_release(BpFootprints* f);

}  // namespace monte
