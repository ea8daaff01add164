// tiles_dispatch.h -- per-n launchers of the tile step, one translation
// unit each (tiles_n<N>.cu), called by the dispatch in tiles.cu.
#pragma once

#include <cuda_runtime.h>

#include <atomic>

#include "geom.cuh"
#include "kernels.cuh"
#include "rows_setup.cuh"
#include "tile_ops.cuh"

namespace faces {

cudaError_t tiles_n2(const FieldDesc &f, const RowPlan &p, long grid, bool general, cudaStream_t s,
                     const PackFuse *fuse);
cudaError_t tiles_n3(const FieldDesc &f, const RowPlan &p, long grid, bool general, cudaStream_t s,
                     const PackFuse *fuse);
cudaError_t tiles_n4(const FieldDesc &f, const RowPlan &p, long grid, bool general, cudaStream_t s,
                     const PackFuse *fuse);
cudaError_t tiles_n5(const FieldDesc &f, const RowPlan &p, long grid, bool general, cudaStream_t s,
                     const PackFuse *fuse);
cudaError_t tiles_n6(const FieldDesc &f, const RowPlan &p, long grid, bool general, cudaStream_t s,
                     const PackFuse *fuse);
cudaError_t tiles_n7(const FieldDesc &f, const RowPlan &p, long grid, bool general, cudaStream_t s,
                     const PackFuse *fuse);
cudaError_t tiles_n8(const FieldDesc &f, const RowPlan &p, long grid, bool general, cudaStream_t s,
                     const PackFuse *fuse);
cudaError_t tiles_n9(const FieldDesc &f, const RowPlan &p, long grid, bool general, cudaStream_t s,
                     const PackFuse *fuse);
cudaError_t tiles_n10(const FieldDesc &f, const RowPlan &p, long grid, bool general, cudaStream_t s,
                     const PackFuse *fuse);
cudaError_t tiles_n11(const FieldDesc &f, const RowPlan &p, long grid, bool general, cudaStream_t s,
                     const PackFuse *fuse);
cudaError_t tiles_n12(const FieldDesc &f, const RowPlan &p, long grid, bool general, cudaStream_t s,
                     const PackFuse *fuse);

cudaError_t wtiles_n2(const FieldDesc &f, const RowPlan &p, long grid, cudaStream_t s);
cudaError_t wtiles_n3(const FieldDesc &f, const RowPlan &p, long grid, cudaStream_t s);
cudaError_t wtiles_n4(const FieldDesc &f, const RowPlan &p, long grid, cudaStream_t s);
cudaError_t wtiles_n5(const FieldDesc &f, const RowPlan &p, long grid, cudaStream_t s);
cudaError_t wtiles_n6(const FieldDesc &f, const RowPlan &p, long grid, cudaStream_t s);
cudaError_t wtiles_n7(const FieldDesc &f, const RowPlan &p, long grid, cudaStream_t s);
cudaError_t wtiles_n8(const FieldDesc &f, const RowPlan &p, long grid, cudaStream_t s);
cudaError_t wtiles_n9(const FieldDesc &f, const RowPlan &p, long grid, cudaStream_t s);
cudaError_t wtiles_n10(const FieldDesc &f, const RowPlan &p, long grid, cudaStream_t s);
cudaError_t wtiles_n11(const FieldDesc &f, const RowPlan &p, long grid, cudaStream_t s);
cudaError_t wtiles_n12(const FieldDesc &f, const RowPlan &p, long grid, cudaStream_t s);

// stages of the tile kernels' cp.async pipeline
constexpr int kTileStages = 3;

// A kernel's dynamic shared-memory limit (cudaFuncSetAttribute) is a
// property of the kernel on one device.  `done` holds one bit per device
// index on which it has been raised to `bytes`; devices 64 and up set it on
// every launch.
inline cudaError_t raise_smem_limit(const void *kernel, int bytes, std::atomic<unsigned long long> &done)
{
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  const unsigned long long bit = dev >= 0 && dev < 64 ? 1ull << dev : 0ull;
  if (bit && (done.load(std::memory_order_acquire) & bit)) return cudaSuccess;
  e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
  if (e == cudaSuccess && bit) done.fetch_or(bit, std::memory_order_acq_rel);
  return e;
}

// the warp-tile form: warps per block, and stages per warp: 3 where a stage
// is at most 8 KB, else 2 (so that blocks of large n still fit several to an
// SM)
constexpr int kWarpsPerBlock = 4;
__host__ __device__ constexpr int wtile_stages(int n)
{
  return (tile_kwarp(n) * n * n * smem_row_stride(n) + 2 * n * n) * 8 <= 8192 ? 3 : 2;
}

// shared memory of the warp-tile form for n (tiles.cu)
size_t wtile_smem_bytes(int n);

}  // namespace faces
