// batch_kernel.h -- the batched tile kernel as used by batches (batch.cu) and
// the job server (serve.cu): a device table of fields and a device work list
// of column units, one persistent launch per share of every listed field.
#pragma once

#include <cuda_runtime.h>

#include <vector>

#include "geom.cuh"
#include "rows_setup.cuh"

namespace faces {

constexpr int kBatchMinN = 2, kBatchMaxN = 10;
// the largest n the warp form of the batched kernel takes (batch_impl.cuh)
constexpr int kBatchWarpMaxN = 5;

struct BatchField {
  FieldDesc f;
  RowPlan p;  // from batch_plan
  int lean;   // 1: the periodic tile step (ptile_steps.cuh), 0: the general one
};

// x-chunks [c0, c1) of one element column of field `field`
struct BatchUnit {
  int field, column, c0, c1;
};

// n the batched kernel handles (direct mode only)
inline bool batch_n_supported(int n) { return n >= kBatchMinN && n <= kBatchMaxN; }

// the tile plan of a field in the batched kernel (half = 1: half-length
// tiles, for the periodic-step form that keeps 4 blocks per SM); lean: the
// field takes the periodic step, whose tiles fill the stage; warp: the field
// takes the warp form (periodic step, n <= kBatchWarpMaxN, half != 1)
RowPlan batch_plan(const FieldDesc &f, int half, bool lean, bool warp = false);

// tile length of the warp form for n
int batch_warp_chunk(int n);

// The launch of a work list whose first nsmall units take the warp form:
// G the blocks that fit, nlarge the other units, *_pts the points of each
// part, boost the warp blocks' weight, run the block pipeline's run length.
// Sets the warp blocks (boost x their share of the points, at least one,
// one or more left for the other units) and the whole grid.
void warp_split(long G, int nsmall, long nlarge, double small_pts, double large_pts, int boost, int run,
                int &wblocks, long &grid);

// resident blocks per SM (3, or 4 with half-length tiles)
int batch_blocks_per_sm(int half = 0);

// sets the kernel's shared-memory attribute on the current device (call once
// per device before the first launch)
cudaError_t batch_configure();

// appends the units of field `field` (column units cut into unit_div parts)
void append_units(std::vector<BatchUnit> &units, int field, const RowPlan &p, int unit_div);

// the kernel form for a field table: 0 all general, 1 all periodic (lean), 2 mixed
int batch_mode(const BatchField *fields, size_t n);

// one share of every field the units cover; blocks take runs of `run`
// consecutive units (block b: runs b, b + grid, ...); half = 1 or 2 only with
// mode 1 and plans from batch_plan(f, half).  The first nsmall units (warp-
// form plans, mode 1, half != 1) go to blocks [0, wblocks), warp by warp;
// the others to the remaining blocks.
cudaError_t launch_batch(const BatchField *d_fields, const BatchUnit *d_units, int nunits, long grid, int run,
                         int mode, int half, cudaStream_t s, int nsmall = 0, int wblocks = 0);

// the kernel's forms, one translation unit each (batch_k<MODE><H>.cu):
// MODE 0 general step, 1 periodic step, 2 each field its own; H the tile
// length form (periodic step only)
cudaError_t batch_configure_00();
cudaError_t batch_configure_20();
cudaError_t batch_configure_10();
cudaError_t batch_configure_11();
cudaError_t batch_configure_12();
cudaError_t batch_launch_00(const BatchField *, const BatchUnit *, int nunits, long grid, int run, int nsmall,
                            int wblocks, cudaStream_t);
cudaError_t batch_launch_20(const BatchField *, const BatchUnit *, int nunits, long grid, int run, int nsmall,
                            int wblocks, cudaStream_t);
cudaError_t batch_launch_10(const BatchField *, const BatchUnit *, int nunits, long grid, int run, int nsmall,
                            int wblocks, cudaStream_t);
cudaError_t batch_launch_11(const BatchField *, const BatchUnit *, int nunits, long grid, int run, int nsmall,
                            int wblocks, cudaStream_t);
cudaError_t batch_launch_12(const BatchField *, const BatchUnit *, int nunits, long grid, int run, int nsmall,
                            int wblocks, cudaStream_t);

}  // namespace faces
