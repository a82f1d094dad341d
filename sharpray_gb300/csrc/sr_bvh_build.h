// sr_bvh_build.h — the binned-SAH BVH build on the device (sr_bvh_build.cu), bit-identical to
// host::build_bvh.
#pragma once

#include <cuda_runtime.h>

#include <vector>

#include "sr_bvh.h"

namespace sr {

// Builds over the shapes' bounds with the reference's parameters (meshes: traverse 1, intersect
// 0.5, 8 bins; scene: 1, 10, 32); `out` receives nodes, items and node count exactly as
// host::build_bvh produces them.  Uses temporary device memory and synchronises `st`.
cudaError_t build_bvh_device(const std::vector<host::Box>& shape_bounds, float cost_traverse, float cost_intersect,
                             int bins, cudaStream_t st, host::BvhHost& out);

}  // namespace sr
