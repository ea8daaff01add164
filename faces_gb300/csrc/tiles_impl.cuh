// tiles_impl.cuh -- the tile-step kernels and their per-n launchers
// (templates).  Each tiles_n<N>.cu instantiates them for one n, so that the
// build compiles the n's in parallel; tiles.cu holds the dispatch on n.
//
// Persistent CTAs walk the tiles of rows_setup.cuh.  Per tile: the staged
// rows arrive by cp.async (three stages: the next two tiles' copies are in
// flight while this one is summed), every owned shared point is summed once from
// shared memory by one thread (tile_ops.cuh), and the changed rows are stored
// back.  Global traffic is one read and one write of every row that holds a
// shared point; the FP64 adds are dense in every warp.
#pragma once

#include <cuda_runtime.h>

#include "geom.cuh"
#include "kernels.cuh"
#include "pack_steps.cuh"
#include "ptile_steps.cuh"
#include "rows_setup.cuh"
#include "tile_ops.cuh"
#include "tile_steps.cuh"
#include "tiles_dispatch.h"
#include "xtile_steps.cuh"

namespace faces {

using namespace tiledev;


template <int N, int K, int NS>
__global__ void __launch_bounds__(256, 3) tile_kernel(FieldDesc f, RowPlan p)
{
  constexpr int NN = N * N, NP = pieces_per_row(N), PW = piece_doubles(N), RS = smem_row_stride(N);
  constexpr int SPT = (NN * NP + 255) / 256;
  constexpr int stage = tile_stage_size<N, K>();
  extern __shared__ __align__(16) double sm[];
  static_assert(stage % 2 == 0, "stages must keep 16-byte alignment");
  double **lop_base = reinterpret_cast<double **>(sm + NS * stage);
  unsigned *rfl_base = reinterpret_cast<unsigned *>(sm + NS * stage + lop_doubles(N, NS));
  SlotCol *rinfo_base = reinterpret_cast<SlotCol *>(sm + NS * stage + lop_doubles(N, NS) + rfl_doubles(N, NS));
  int4 *tinfo = reinterpret_cast<int4 *>(sm + NS * stage + lop_doubles(N, NS) + rfl_doubles(N, NS) +
                                         rinfo_doubles(N, NS));
  static_assert(sizeof(SlotCol) == 16, "row info is two doubles");

  // The block's tiles, walked by a TileWalk: a contiguous range (order 1),
  // every gridDim.x-th tile (order 0), or every gridDim.x-th unit of
  // unit_chunks consecutive chunks of one column, units ordered chunk group
  // first so that the blocks running at one time hold neighbouring columns
  // (order 2).  Consecutive tiles of one column share their rows' sources.
  TileWalk nw;  // next tile to stage
  walk_begin(p, nw);
  if (nw.done) return;
  int inflight = 0;  // staged tiles not yet summed
  ColKey ck{};
  bool have_col = false;
  SlotCol col[SPT];  // the staged column's row sources, per owned slot
#pragma unroll
  for (int j = 0; j < NS - 1; j++) {
    if (!nw.done) {
      stage_tile<N, K, SPT>(f, p, nw.u, ck, have_col, col, sm + j * stage, rfl_base + j * NN, lop_base + j * NN,
                            rinfo_base + j * NN, tinfo + j);
      walk_next(p, nw);
      inflight++;
    } else {
      cp_commit();
    }
  }
  // the loop reads row flags and tile infos other threads wrote
  __syncthreads();
  int s = 0;
  for (; inflight > 0; inflight--) {
    cp_wait<NS - 2>();
    const unsigned *rfl = rfl_base + s * NN;
    const int4 ti = tinfo[s];
    const int nk = ti.y;
    const bool hx = ti.z != 0;
    bool ok = true;
    if ((int)threadIdx.x < NN) ok = row_regular(rfl[threadIdx.x], hx);
    const int regular = __syncthreads_and(ok);
    // the stage of the previous tile is free again: the next prefetch goes there
    const int sn = (s + NS - 1) % NS;
    if (!nw.done) {
      stage_tile<N, K, SPT>(f, p, nw.u, ck, have_col, col, sm + sn * stage, rfl_base + sn * NN, lop_base + sn * NN,
                            rinfo_base + sn * NN, tinfo + sn);
      walk_next(p, nw);
      inflight++;
    } else {
      cp_commit();
    }
    double *buf = sm + s * stage;
    if (nk > 0) sum_tile<N, K>(buf, rfl, nk, hx, regular != 0);
    __syncthreads();
    if (nk > 0) store_tile<N, K, SPT>(buf, rfl, lop_base + s * NN, rinfo_base + s * NN, ti.x, nk, hx);
    s = (s + 1) % NS;
  }
}

// The periodic tile step (ptile_steps.cuh): the same pipeline with row
// sources computed from four column offsets per tile.
template <int N, int K, int NS>
__global__ void __launch_bounds__(256, 4) ptile_kernel(FieldDesc f, RowPlan p)
{
  constexpr int stage = tile_stage_size<N, K>();
  extern __shared__ __align__(16) double sm[];
  static_assert(stage % 2 == 0, "stages must keep 16-byte alignment");
  PMeta *meta = reinterpret_cast<PMeta *>(sm + NS * stage);
  int4 *tinfo = reinterpret_cast<int4 *>(meta + NS);
  TileWalk nw;
  walk_begin(p, nw);
  if (nw.done) return;
  int inflight = 0;
#pragma unroll
  for (int j = 0; j < NS - 1; j++) {
    if (!nw.done) {
      ptile::pstage<N, K>(f, p, nw.u, sm + j * stage, meta + j, tinfo + j, threadIdx.x);
      walk_next(p, nw);
      inflight++;
    } else {
      cp_commit();
    }
  }
  int s = 0;
  for (; inflight > 0; inflight--) {
    cp_wait<NS - 2>();
    // the staged tile, its infos, and the end of the previous tile's store
    __syncthreads();
    const int nk = tinfo[s].y;
    const int sn = (s + NS - 1) % NS;
    if (!nw.done) {
      ptile::pstage<N, K>(f, p, nw.u, sm + sn * stage, meta + sn, tinfo + sn, threadIdx.x);
      walk_next(p, nw);
      inflight++;
    } else {
      cp_commit();
    }
    double *buf = sm + s * stage;
    ptile::pxpass<N, K>(f.u, buf, meta + s, nk, threadIdx.x);
    __syncthreads();
    ptile::pyzpass<N, K>(f.u, buf, meta + s, nk, threadIdx.x);
    s = (s + 1) % NS;
  }
}

// The message-mode tile step (xtile_steps.cuh): the periodic step's
// pipeline, with remote rows and x ends read from the received messages and
// only the rank's own copies stored.  Tile i is described (addresses, from
// the receive table) in iteration i-3, staged in iteration i-2 and summed in
// iteration i: NS data stages and NS+1 records, two block barriers per tile.
// The fused pack's wait: thread 0 of a block polls the arrival counter
// (acquire loads, short sleeps) until every block of the launch has packed,
// at most pf.polls times; a wait that runs out sets bit 0 of *err and lets
// the block go on (its results are then not to be trusted: the host reads the
// flag with faces_status).

__device__ __forceinline__ unsigned long long pack_arrivals(const unsigned long long *counter)
{
  unsigned long long v;
  asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(counter) : "memory");
  return v;
}

__device__ __forceinline__ void pack_wait(const PackFuse &pf, unsigned long long blocks)
{
  for (long i = 0; pack_arrivals(pf.counter) < blocks; i++) {
    if (i >= pf.polls) {
      atomicOr(pf.err, 1);
      return;
    }
    __nanosleep(64);
  }
}

template <int N, int K, int NS, bool OPEN, bool FUSE>
__global__ void __launch_bounds__(256, 4) xtile_kernel(FieldDesc f, RowPlan p, PackFuse pf)
{
  constexpr int stage = tile_stage_size<N, K>();
  constexpr int NR = NS + 1;
  extern __shared__ __align__(16) double sm[];
  static_assert(stage % 2 == 0, "stages must keep 16-byte alignment");
  static_assert(sizeof(XMeta) % 16 == 0, "tile records keep 16-byte alignment");
  XMeta *rec = reinterpret_cast<XMeta *>(sm + NS * stage);
  const int t = threadIdx.x;
  if constexpr (FUSE) {
    // the pack: this block's share of its blocks, then its arrival (every
    // block arrives once, whether or not it has tiles)
    const long pb = (long)pf.gx * pf.gy;
    for (long v = blockIdx.x; v < pb; v += gridDim.x) {
      const int vx = (int)(v % pf.gx), vy = (int)(v / pf.gx);
      if (pf.wide) pack_block<unsigned long>(f, vy, vx, pf.gx, t, 256);
      else pack_block<unsigned>(f, vy, vx, pf.gx, t, 256);
    }
    __syncthreads();
    if (t == 0) {
      __threadfence();
      atomicAdd(pf.counter, 1ULL);
    }
  }
  // Before a tile that reads a message or writes a boundary point is
  // staged, every block must have packed (block-uniform: the record is in
  // shared memory); interior tiles run beside other blocks' packing.
  bool packed = !FUSE;
  auto ready = [&](const XMeta *r) {
    if (FUSE && !packed && !xtile::interior(r)) {
      if (t == 0) pack_wait(pf, gridDim.x + (unsigned)pf.extra);
      __syncthreads();
      (void)pack_arrivals(pf.counter);  // every thread's own acquire
      packed = true;
    }
  };
  TileWalk nw;
  walk_begin(p, nw);
  if (nw.done) return;
  int ndesc = 0;  // tiles described so far
  for (int j = 0; j < NR - 1 && !nw.done; j++) {
    xtile::xdescribe<N, OPEN, 256>(f, p, nw.u, rec + j, t);
    walk_next(p, nw);
    ndesc++;
  }
  __syncthreads();
#pragma unroll
  for (int j = 0; j < NS - 1; j++) {
    if (j < ndesc) {
      ready(rec + j);
      xtile::xcopies<N, K, OPEN>(rec + j, sm + j * stage, t);
    } else {
      cp_commit();
    }
  }
  for (int i = 0; i < ndesc; i++) {
    cp_wait<NS - 2>();
    // tile i's stage, the records up to i+NS-1, and the end of tile i-1's
    // stores (its stage and record are free again)
    __syncthreads();
    if (i + NS - 1 < ndesc) {
      ready(rec + (i + NS - 1) % NR);
      xtile::xcopies<N, K, OPEN>(rec + (i + NS - 1) % NR, sm + ((i + NS - 1) % NS) * stage, t);
    } else {
      cp_commit();
    }
    double *buf = sm + (i % NS) * stage;
    const XMeta *r = rec + i % NR;
    // an open field's tiles away from its boundary are complete: they take
    // the passes' periodic form (block-uniform)
    const bool full = xtile::complete<OPEN>(r);
    if (full) xtile::xxpass<N, K, false>(buf, r, t);
    else xtile::xxpass<N, K, OPEN>(buf, r, t);
    if (!nw.done) {
      xtile::xdescribe<N, OPEN, 256>(f, p, nw.u, rec + (i + NR - 1) % NR, t);
      walk_next(p, nw);
      ndesc++;
    }
    __syncthreads();
    if (full) xtile::xyzpass<N, K, false>(buf, r, t);
    else xtile::xyzpass<N, K, OPEN>(buf, r, t);
  }
}

// The warp-tile form of the periodic step: every warp stages, sums and
// stores its own tiles (tile_kwarp(n) elements, wtile_stages(n) stages), so a
// block holds kWarpsPerBlock independent pipelines and needs no block
// barrier; warps walk the tiles chunk group first (tile q: chunk q / columns,
// column q % columns) with a stride of all warps of the grid.
template <int N, int K, int NS, int WPB>
__global__ void __launch_bounds__(WPB * 32) wtile_kernel(FieldDesc f, RowPlan p)
{
  constexpr int stage = tile_stage_size<N, K>();
  extern __shared__ __align__(16) double sm[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  double *wsm = sm + (long)warp * NS * stage;
  PMeta *meta_all = reinterpret_cast<PMeta *>(sm + (long)WPB * NS * stage);
  PMeta *meta = meta_all + warp * NS;
  int4 *tinfo = reinterpret_cast<int4 *>(meta_all + WPB * NS) + warp * NS;
  const int ncol = (int)(p.ntiles / p.nchunks), total = (int)p.ntiles;
  const int stride = gridDim.x * WPB;
  int q = blockIdx.x * WPB + warp;  // next tile to stage
  auto cursor = [&](int t) {
    TileCursor u;
    u.c = t / ncol;
    const int col = t - u.c * ncol, t2 = col / p.ty;
    u.jy = col - t2 * p.ty;
    u.jz = t2 % p.tz;
    u.r = t2 / p.tz;
    return u;
  };
  int inflight = 0;
#pragma unroll
  for (int j = 0; j < NS - 1; j++) {
    if (q < total) {
      ptile::pstage<N, K, 32>(f, p, cursor(q), wsm + j * stage, meta + j, tinfo + j, lane);
      q += stride;
      inflight++;
    } else {
      cp_commit();
    }
  }
  int s = 0;
  for (; inflight > 0; inflight--) {
    cp_wait<NS - 2>();
    // the staged tile and its infos, and the end of the previous tile's work
    __syncwarp();
    const int nk = tinfo[s].y;
    const int sn = (s + NS - 1) % NS;
    if (q < total) {
      ptile::pstage<N, K, 32>(f, p, cursor(q), wsm + sn * stage, meta + sn, tinfo + sn, lane);
      q += stride;
      inflight++;
    } else {
      cp_commit();
    }
    double *buf = wsm + s * stage;
    ptile::pxpass<N, K, 32>(f.u, buf, meta + s, nk, lane);
    __syncwarp();
    ptile::pyzpass<N, K, 32>(f.u, buf, meta + s, nk, lane);
    s = (s + 1) % NS;
  }
}

// The mixed tile step for fields the periodic step does not take (open
// fields, v-26 messages): per tile, block-uniformly, interior tiles
// (interior_tile) take the periodic step's staging and passes, the others
// the general step's.  Shared memory holds both layouts' per-stage records.
template <int N, int K, int NS>
__global__ void __launch_bounds__(256, 3) mtile_kernel(FieldDesc f, RowPlan p)
{
  constexpr int NN = N * N, NP = pieces_per_row(N);
  constexpr int SPT = (NN * NP + 255) / 256;
  constexpr int stage = tile_stage_size<N, K>();
  extern __shared__ __align__(16) double sm[];
  double **lop_base = reinterpret_cast<double **>(sm + NS * stage);
  unsigned *rfl_base = reinterpret_cast<unsigned *>(sm + NS * stage + lop_doubles(N, NS));
  SlotCol *rinfo_base = reinterpret_cast<SlotCol *>(sm + NS * stage + lop_doubles(N, NS) + rfl_doubles(N, NS));
  int4 *tinfo = reinterpret_cast<int4 *>(sm + NS * stage + lop_doubles(N, NS) + rfl_doubles(N, NS) +
                                         rinfo_doubles(N, NS));
  PMeta *meta = reinterpret_cast<PMeta *>(tinfo + NS);
  TileWalk nw;
  walk_begin(p, nw);
  if (nw.done) return;
  int inflight = 0;
  ColKey ck{};
  bool have_col = false;
  SlotCol col[SPT];
  // stage the next tile into stage st; the tile info's z: bit 0 hi_x, bit 1
  // the periodic step
  auto stage_next = [&](int st) {
    if (interior_tile(f, p.nchunks, nw.u.c, nw.u.jy, nw.u.jz)) {
      ptile::pstage<N, K>(f, p, nw.u, sm + st * stage, meta + st, tinfo + st, threadIdx.x);
      if (threadIdx.x == 0) tinfo[st].z = 2;
    } else {
      stage_tile<N, K, SPT>(f, p, nw.u, ck, have_col, col, sm + st * stage, rfl_base + st * NN, lop_base + st * NN,
                            rinfo_base + st * NN, tinfo + st);
    }
    walk_next(p, nw);
    inflight++;
  };
#pragma unroll
  for (int j = 0; j < NS - 1; j++) {
    if (!nw.done) stage_next(j);
    else cp_commit();
  }
  __syncthreads();
  int s = 0;
  for (; inflight > 0; inflight--) {
    cp_wait<NS - 2>();
    const unsigned *rfl = rfl_base + s * NN;
    const int4 ti = tinfo[s];
    const int nk = ti.y;
    const bool hx = (ti.z & 1) != 0, lean = (ti.z & 2) != 0;
    bool ok = true;
    if (!lean && (int)threadIdx.x < NN) ok = row_regular(rfl[threadIdx.x], hx);
    const int regular = __syncthreads_and(ok);
    const int sn = (s + NS - 1) % NS;
    if (!nw.done) stage_next(sn);
    else cp_commit();
    double *buf = sm + s * stage;
    if (nk > 0) {
      if (lean) ptile::pxpass<N, K>(f.u, buf, meta + s, nk, threadIdx.x);
      else sum_tile<N, K>(buf, rfl, nk, hx, regular != 0);
    }
    __syncthreads();
    if (nk > 0) {
      if (lean) ptile::pyzpass<N, K>(f.u, buf, meta + s, nk, threadIdx.x);
      else store_tile<N, K, SPT>(buf, rfl, lop_base + s * NN, rinfo_base + s * NN, ti.x, nk, hx);
    }
    s = (s + 1) % NS;
  }
}

template <int N>
inline cudaError_t launch_wtiles_n(const FieldDesc &f, const RowPlan &p, long grid, cudaStream_t s)
{
  constexpr int K = tile_kwarp(N);
  if (p.chunk > K) return cudaErrorInvalidValue;
  const size_t smem = wtile_smem_bytes(N);
  static std::atomic<unsigned long long> configured{0};
  if (cudaError_t e = raise_smem_limit((const void *)wtile_kernel<N, K, wtile_stages(N), kWarpsPerBlock>, (int)smem,
                                       configured))
    return e;
  long blocks = (p.ntiles + kWarpsPerBlock - 1) / kWarpsPerBlock;
  if (grid < blocks) blocks = grid;
  if (blocks < 1) return cudaSuccess;
  wtile_kernel<N, K, wtile_stages(N), kWarpsPerBlock><<<(unsigned)blocks, 32 * kWarpsPerBlock, smem, s>>>(f, p);
  return cudaGetLastError();
}

// The message-mode step with the pack in its prologue: one cooperative
// launch (every block resident, so that a block's wait for the others ends),
// the grid capped at what is resident, the arrival counter zeroed first.
template <int N, int K, bool OPEN>
inline cudaError_t launch_xtile_fused(const FieldDesc &f, const RowPlan &p, long grid, size_t smem,
                                      const PackFuse &pf, cudaStream_t s)
{
  const void *kern = (const void *)xtile_kernel<N, K, kTileStages, OPEN, true>;
  static std::atomic<unsigned long long> configured{0};
  if (cudaError_t e = raise_smem_limit(kern, (int)smem, configured)) return e;
  // the resident blocks of the whole device, found once per device
  static std::atomic<long> resident[64];
  int dev = 0;
  cudaError_t e;
  if ((e = cudaGetDevice(&dev)) != cudaSuccess) return e;
  long cap = dev >= 0 && dev < 64 ? resident[dev].load() : 0;
  if (cap <= 0) {
    int sms = 0, per_sm = 0;
    if ((e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess ||
        (e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, 256, smem)) != cudaSuccess)
      return e;
    cap = (long)per_sm * sms;
    if (dev >= 0 && dev < 64) resident[dev].store(cap);
  }
  if (grid > cap) grid = cap;
  if (grid < 1) return cudaErrorCooperativeLaunchTooLarge;
  if ((e = cudaMemsetAsync(pf.counter, 0, sizeof(unsigned long long), s)) != cudaSuccess) return e;
  FieldDesc fa = f;
  RowPlan pa = p;
  PackFuse pfa = pf;
  void *args[] = {&fa, &pa, &pfa};
  return cudaLaunchCooperativeKernel(kern, dim3((unsigned)grid), dim3(256), args, smem, s);
}

template <int N, int K>
inline cudaError_t launch_tiles_nk(const FieldDesc &f, const RowPlan &p, long grid, bool general, cudaStream_t s,
                                   const PackFuse *fuse)
{
  static_assert(tile_stage_size<N, K>() * sizeof(double) % 16 == 0, "stage alignment");
  if (grid > p.ntiles) grid = p.ntiles;
  if (grid < 1) return cudaSuccess;
  if (!general && xtile_field(f)) {
    const size_t smem = sizeof(double) * kTileStages * tile_stage_size<N, K>() + sizeof(XMeta) * (kTileStages + 1);
    if (fuse && f.mode == kMessages) {
      if (f.periodic) return launch_xtile_fused<N, K, false>(f, p, grid, smem, *fuse, s);
      return launch_xtile_fused<N, K, true>(f, p, grid, smem, *fuse, s);
    }
    const PackFuse none{};
    if (f.periodic) {
      static std::atomic<unsigned long long> configured{0};
      if (cudaError_t e =
              raise_smem_limit((const void *)xtile_kernel<N, K, kTileStages, false, false>, (int)smem, configured))
        return e;
      xtile_kernel<N, K, kTileStages, false, false><<<(unsigned)grid, 256, smem, s>>>(f, p, none);
    } else {
      static std::atomic<unsigned long long> configured{0};
      if (cudaError_t e =
              raise_smem_limit((const void *)xtile_kernel<N, K, kTileStages, true, false>, (int)smem, configured))
        return e;
      xtile_kernel<N, K, kTileStages, true, false><<<(unsigned)grid, 256, smem, s>>>(f, p, none);
    }
  } else if (!general && !ptile_field(f)) {
    const size_t smem = tile_smem_bytes(N, K) + sizeof(PMeta) * kTileStages;
    static std::atomic<unsigned long long> configured{0};
    if (cudaError_t e = raise_smem_limit((const void *)mtile_kernel<N, K, kTileStages>, (int)smem, configured)) return e;
    mtile_kernel<N, K, kTileStages><<<(unsigned)grid, 256, smem, s>>>(f, p);
  } else if (general) {
    const size_t smem = tile_smem_bytes(N, K);
    static std::atomic<unsigned long long> configured{0};
    if (cudaError_t e = raise_smem_limit((const void *)tile_kernel<N, K, kTileStages>, (int)smem, configured)) return e;
    tile_kernel<N, K, kTileStages><<<(unsigned)grid, 256, smem, s>>>(f, p);
  } else {
    const size_t smem = sizeof(double) * kTileStages * tile_stage_size<N, K>() +
                        (sizeof(PMeta) + sizeof(int4)) * kTileStages;
    static std::atomic<unsigned long long> configured{0};
    if (cudaError_t e = raise_smem_limit((const void *)ptile_kernel<N, K, kTileStages>, (int)smem, configured)) return e;
    ptile_kernel<N, K, kTileStages><<<(unsigned)grid, 256, smem, s>>>(f, p);
  }
  return cudaGetLastError();
}

template <int N>
inline cudaError_t launch_tiles_n(const FieldDesc &f, const RowPlan &p, long grid, bool general, cudaStream_t s,
                                  const PackFuse *fuse)
{
  constexpr int KM = tile_kinst_max(N);
  if (p.chunk > KM) return cudaErrorInvalidValue;
  switch (tile_instance_k(p.chunk)) {
    case 1: return launch_tiles_nk<N, 1>(f, p, grid, general, s, fuse);
    case 2: return launch_tiles_nk<N, 2>(f, p, grid, general, s, fuse);
    case 4: return launch_tiles_nk<N, 4>(f, p, grid, general, s, fuse);
    case 8: return launch_tiles_nk<N, 8>(f, p, grid, general, s, fuse);
    case 16:
      if constexpr (KM >= 16) return launch_tiles_nk<N, 16>(f, p, grid, general, s, fuse);
      return cudaErrorInvalidValue;
    case 32:
      if constexpr (KM >= 32) return launch_tiles_nk<N, 32>(f, p, grid, general, s, fuse);
      return cudaErrorInvalidValue;
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace faces
