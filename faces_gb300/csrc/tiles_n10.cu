// tiles_n10.cu -- the tile-step kernels for n = 10 (tiles_impl.cuh).
#include "tiles_impl.cuh"

namespace faces {

cudaError_t tiles_n10(const FieldDesc &f, const RowPlan &p, long grid, bool general, cudaStream_t s,
                     const PackFuse *fuse)
{
  return launch_tiles_n<10>(f, p, grid, general, s, fuse);
}

cudaError_t wtiles_n10(const FieldDesc &f, const RowPlan &p, long grid, cudaStream_t s)
{
  return launch_wtiles_n<10>(f, p, grid, s);
}

}  // namespace faces
