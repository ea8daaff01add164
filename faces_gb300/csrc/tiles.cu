// tiles.cu -- the tile step's host side: which kernel instance runs (the
// dispatch on n to tiles_n<N>.cu, whose kernels are in tiles_impl.cuh), the
// default tile length, and the shared memory and resident blocks per SM of
// each form.
#include <cuda_runtime.h>

#include "kernels.cuh"
#include "ptile_steps.cuh"
#include "tile_ops.cuh"
#include "tile_steps.cuh"
#include "tiles_dispatch.h"
#include "xtile_steps.cuh"

namespace faces {

bool tile_kernel_supported(int n) { return n >= 2 && n <= 12; }

int tile_default_chunk(int n) { return tile_kmax(n); }

// The periodic and message-mode steps run faster with the longest tile that
// still leaves two blocks per SM (at most 110 KB of shared memory) than with
// ~20 KB stages: measured on 95x94x93 n = 12 (2 elements: 4.37 vs 4.84 ms per
// share periodic, 4.93 vs 5.34 open), 48^3 n = 10 (4: 0.312 vs 0.337), 40^3
// n = 11 (2: 0.276 vs 0.287), 48^3 n = 9 (4: 0.240 vs 0.261), 56^3 n = 7 (8:
// 0.213 vs 0.278), 60^3 n = 5 (16: 0.112 vs 0.126); n = 6 and 8 keep their
// lengths (8 and 4).  Small fields shorten it again (faces_api.cu).
int tile_default_chunk(int n, TileForm form)
{
  if (form == kGeneralForm) return tile_kmax(n);
  int k = 1;
  while (k * 2 <= tile_kinst_max(n) && tile_form_smem_bytes(n, k * 2, form) <= 110 * 1024) k *= 2;
  return k;
}

size_t tile_smem_bytes(int n, int chunk)
{
  const int K = tile_instance_k(chunk);
  // data stages, x-lower pointers, row flags, tile infos (see tile_kernel)
  return sizeof(double) * (kTileStages * tile_stage_doubles(n, K) + lop_doubles(n, kTileStages) +
                           rfl_doubles(n, kTileStages) + rinfo_doubles(n, kTileStages)) +
         sizeof(int4) * kTileStages;
}

TileForm tile_form(const FieldDesc &f, bool general)
{
  if (!general && xtile_field(f)) return kExchangeForm;
  if (!general && ptile_field(f)) return kPeriodicForm;
  return kGeneralForm;
}

// resident blocks per SM: shared memory (228 KB per SM, 1 KB reserved per
// block) and the launch bounds' register budget (general 3, periodic and
// message-mode 4)
size_t tile_form_smem_bytes(int n, int chunk, TileForm form)
{
  const int K = tile_instance_k(chunk);
  const size_t data = sizeof(double) * kTileStages * tile_stage_doubles(n, K);
  return form == kPeriodicForm   ? data + (sizeof(PMeta) + sizeof(int4)) * kTileStages
         : form == kExchangeForm ? data + sizeof(XMeta) * (kTileStages + 1)
                                 : tile_smem_bytes(n, chunk);
}

int tile_blocks_per_sm(int n, int chunk, TileForm form)
{
  const size_t smem = tile_form_smem_bytes(n, chunk, form);
  int fit = (int)((228 * 1024) / (smem + 1024));
  const int regs_fit = form == kGeneralForm ? 3 : 4;
  return fit < 1 ? 1 : fit > regs_fit ? regs_fit : fit;
}

size_t wtile_smem_bytes(int n)
{
  return sizeof(double) * kWarpsPerBlock * wtile_stages(n) * tile_stage_doubles(n, tile_kwarp(n)) +
         (sizeof(PMeta) + sizeof(int4)) * kWarpsPerBlock * wtile_stages(n);
}

int wtile_blocks_per_sm(int n)
{
  const int fit = (int)((228 * 1024) / (wtile_smem_bytes(n) + 1024));
  return fit < 1 ? 1 : fit > 16 ? 16 : fit;
}

cudaError_t launch_wtiles(const FieldDesc &f, const RowPlan &p, long grid, cudaStream_t s)
{
  if (!ptile_field(f)) return cudaErrorInvalidValue;
  switch (f.n) {
    case 2: return wtiles_n2(f, p, grid, s);
    case 3: return wtiles_n3(f, p, grid, s);
    case 4: return wtiles_n4(f, p, grid, s);
    case 5: return wtiles_n5(f, p, grid, s);
    case 6: return wtiles_n6(f, p, grid, s);
    case 7: return wtiles_n7(f, p, grid, s);
    case 8: return wtiles_n8(f, p, grid, s);
    case 9: return wtiles_n9(f, p, grid, s);
    case 10: return wtiles_n10(f, p, grid, s);
    case 11: return wtiles_n11(f, p, grid, s);
    case 12: return wtiles_n12(f, p, grid, s);
    default: return cudaErrorInvalidValue;
  }
}

cudaError_t launch_tiles(const FieldDesc &f, const RowPlan &p, long grid, cudaStream_t s, bool general,
                         const PackFuse *fuse)
{
  switch (f.n) {
    case 2: return tiles_n2(f, p, grid, general, s, fuse);
    case 3: return tiles_n3(f, p, grid, general, s, fuse);
    case 4: return tiles_n4(f, p, grid, general, s, fuse);
    case 5: return tiles_n5(f, p, grid, general, s, fuse);
    case 6: return tiles_n6(f, p, grid, general, s, fuse);
    case 7: return tiles_n7(f, p, grid, general, s, fuse);
    case 8: return tiles_n8(f, p, grid, general, s, fuse);
    case 9: return tiles_n9(f, p, grid, general, s, fuse);
    case 10: return tiles_n10(f, p, grid, general, s, fuse);
    case 11: return tiles_n11(f, p, grid, general, s, fuse);
    case 12: return tiles_n12(f, p, grid, general, s, fuse);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace faces
