// kernels.cuh -- launch wrappers for the sm_103a halo-sum kernels.
#pragma once

#include <cuda_runtime.h>

#include "geom.cuh"
#include "rows_setup.cuh"

namespace faces {

bool row_kernel_supported(int n);

cudaError_t launch_init_ref(const FieldDesc &f, cudaStream_t s);
cudaError_t launch_init_int(const FieldDesc &f, unsigned long long seed, cudaStream_t s);
cudaError_t launch_pack(const FieldDesc &f, cudaStream_t s);
cudaError_t launch_gather(const FieldDesc &f, int compute, cudaStream_t s);
cudaError_t launch_rows(const FieldDesc &f, const RowPlan &p, cudaStream_t s);

// seam step (seams.cu, seam_steps.cuh): direct mode, compute = true; the
// chunked form (chunks of `chunk` elements along x, `grid` blocks) or the
// lean form
struct SeamPlan {
  int chunk, nch;
  long units, plane_items, grid;
  int lean;  // the lean form: a thread per face slot (and the boundary planes' launch)
};
bool seam_kernel_supported(int n);
int seam_default_chunk(int n);
int seam_blocks_per_sm(int n);
SeamPlan make_seam_plan(const FieldDesc &f, int chunk, long grid, int lean);
cudaError_t launch_seams(const FieldDesc &f, const SeamPlan &p, cudaStream_t s);

// v-6 strategy (FACES_V6): six face messages per rank in `msg`
// (v6_message_doubles of them), sweeps z, y, x; six launches
long v6_message_doubles(const FieldDesc &f);
cudaError_t launch_v6(const FieldDesc &f, double *msg, int compute, cudaStream_t s);
// its fused form (FACES_V6F; v6_steps.cuh): four launches, same messages and sums
cudaError_t launch_v6_fused(const FieldDesc &f, double *msg, int compute, cudaStream_t s);

// shared-memory tile step (tiles.cu): chunk (plan.chunk) at most tile_kinst_max(n)
bool tile_kernel_supported(int n);
int tile_default_chunk(int n);
size_t tile_smem_bytes(int n, int chunk);
// which tile kernel a field runs (launch_tiles): the general step (or the
// mixed one), the periodic direct step, or the message-mode step
enum TileForm : int { kGeneralForm = 0, kPeriodicForm = 1, kExchangeForm = 2 };
TileForm tile_form(const FieldDesc &f, bool general);
int tile_blocks_per_sm(int n, int chunk, TileForm form);
// shared memory of one block of a tile form
size_t tile_form_smem_bytes(int n, int chunk, TileForm form);
// the default tile length of a form
int tile_default_chunk(int n, TileForm form);
// the warp-tile form of the periodic step (periodic direct-mode fields; plan
// chunk at most tile_kwarp(n)); grid in blocks of 4 warps
size_t wtile_smem_bytes(int n);
int wtile_blocks_per_sm(int n);
cudaError_t launch_wtiles(const FieldDesc &f, const RowPlan &p, long grid, cudaStream_t s);

// periodic direct-mode fields take the periodic tile step, other fields the
// mixed step (periodic step on interior tiles), unless `general`
// The pack fused into the message-mode tile kernel's prologue: every block
// packs its share of the pack's blocks (pack_steps.cuh, grid gx x gy), then
// adds one to *counter; a tile that reads a message or writes a point the
// pack reads first waits (bounded) until all blocks have; a wait that runs
// out sets bit 0 of *err.  The launch is cooperative (all blocks resident)
// and zeroes *counter before it.
struct PackFuse {
  int gx, gy, wide;
  unsigned long long *counter;
  int *err;
  int extra;   // arrivals waited for beyond the launch's blocks (0; a test sets 1)
  long polls;  // the wait's bound (polls of about 64 ns or more)
};
cudaError_t launch_tiles(const FieldDesc &f, const RowPlan &p, long grid, cudaStream_t s, bool general = false,
                         const PackFuse *fuse = nullptr);

// Closed-form check of a field after `nshares` shares of a known initial
// state (init: 0 = reference formula, 1 = integer seed) with the relative
// error rule of gpu/main.cc:39-105.  Pass 1 (target = 0) raises rank_max[r]
// (per-rank maximum error as an ordered 64-bit pattern; zeroed by the
// caller) and *gmax.  Pass 2 (target = the maximum's pattern) lowers *first
// (set to ~0 by the caller) to the first linear point index with that error.
// Pass 3 (only >= 0) writes (u, expected) of point `only` into vals[2].
// Linear point index = ((((r*mz + jz)*my + jy)*mx + jx)*n + iz)*n*n + iy*n + ix.
cudaError_t launch_check(const FieldDesc &f, int init, unsigned long long seed, int nshares, int compute,
                         unsigned long long *rank_max, unsigned long long *gmax, unsigned long long target,
                         unsigned long long *first, long only, double *vals, cudaStream_t s);

}  // namespace faces
