// query.cuh -- launchers of the all-hits query and the voxel grid.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <string>

#include "../../include/j3dg.h"

namespace j3dg {

struct DevInst;

struct VoxParams {
  float mn[3], mx[3];   // mesh bbox
  uint32_t dim[3];      // voxel grid
  uint32_t rays[3];     // rays of each sweep: dim[(d+1)%3] * dim[(d+2)%3]
  uint32_t rays_total;
  uint32_t use_texture, use_colors;
};

cudaError_t launch_find_all(const DevInst* inst, const j3dg_ray* rays, uint32_t n, uint32_t cap, j3dg_hit* hits,
                            uint32_t* counts, uint32_t* status, cudaStream_t st);
cudaError_t launch_voxelize(const DevInst* inst, const VoxParams& V, uint32_t* keys, uint8_t* out, uint32_t* status,
                            cudaStream_t st);

// Device addresses of the file-scope scratch of the no-allocation voxel grid
// (keys: J3DG_NOALLOC_MAX_VOXELS words; staging: as many bytes), looked up
// with cudaGetSymbolAddress on the current device (contexts do this once,
// when they are created).
int voxel_scratch(uint32_t** keys, uint8_t** staging, std::string& err);

cudaError_t launch_count_hits(const j3dg_pixel* G, size_t n, unsigned long long* out, cudaStream_t st);

}  // namespace j3dg
