// tile_steps.cuh -- device building blocks of the shared-memory tile step:
// staging a tile by cp.async, summing it, storing it back.  Used by the
// single-field kernel (tiles.cu) and the batched kernel (batch.cu).
#pragma once

#include <cuda_runtime.h>

#include "geom.cuh"
#include "rows_setup.cuh"
#include "tile_ops.cuh"

namespace faces {

namespace tiledev {

// host replay: 16-byte copies whose addresses are not both 16-byte aligned
// (on the device such a cp.async faults); the replay requires none
inline long &host_misaligned_copies()
{
  static long count = 0;
  return count;
}

// The host versions serve the CPU replay of the periodic step
// (tests/native/ptile_emu.cu): a copy is done at once, groups are no-ops.
__host__ __device__ __forceinline__ void cp_async(double *dst, const double *src, int len)
{
#ifdef __CUDA_ARCH__
  const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
  if (len == 2)
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(d), "l"(src) : "memory");
  else
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(d), "l"(src) : "memory");
#else
  if (len == 2 && ((reinterpret_cast<unsigned long>(dst) | reinterpret_cast<unsigned long>(src)) & 15))
    host_misaligned_copies()++;
  for (int i = 0; i < len; i++) dst[i] = src[i];
#endif
}

__host__ __device__ __forceinline__ void cp_commit()
{
#ifdef __CUDA_ARCH__
  asm volatile("cp.async.commit_group;" ::: "memory");
#endif
}

template <int W>
__host__ __device__ __forceinline__ void cp_wait()
{
#ifdef __CUDA_ARCH__
  asm volatile("cp.async.wait_group %0;" ::"n"(W) : "memory");
#endif
}

struct ColKey {
  int r, jy, jz;
  bool skip, has_hi;
};

// the sequence of tiles one block processes
struct TileWalk {
  TileCursor u;   // current tile
  long t, t1;     // orders 0/1: tile index and end
  long v, nv;     // order 2: unit index and count
  int c1;         // order 2: end chunk of the unit
  bool done;
};

__device__ __forceinline__ void walk_unit(const RowPlan &p, TileWalk &w)
{
  // unit v: chunk group q = v / columns, column = v % columns
  const long ncol = p.ntiles / p.nchunks;
  const long q = w.v / ncol, column = w.v - q * ncol;
  const int c0 = (int)q * p.unit_chunks;
  w.c1 = min(c0 + p.unit_chunks, p.nchunks);
  w.u = cursor_of(p, column * p.nchunks + c0);
}

__device__ __forceinline__ void walk_begin(const RowPlan &p, TileWalk &w)
{
  w.done = false;
  if (p.order == 2) {
    const long ncol = p.ntiles / p.nchunks;
    w.nv = ncol * ((p.nchunks + p.unit_chunks - 1) / p.unit_chunks);
    w.v = blockIdx.x;
    if (w.v >= w.nv) { w.done = true; return; }
    walk_unit(p, w);
  } else if (p.order == 1) {
    w.t = p.ntiles * blockIdx.x / gridDim.x;
    w.t1 = p.ntiles * (blockIdx.x + 1) / gridDim.x;
    if (w.t >= w.t1) { w.done = true; return; }
    w.u = cursor_of(p, w.t);
  } else {
    w.t = blockIdx.x;
    w.t1 = p.ntiles;
    if (w.t >= w.t1) { w.done = true; return; }
    w.u = cursor_of(p, w.t);
  }
}

__device__ __forceinline__ void walk_next(const RowPlan &p, TileWalk &w)
{
  if (p.order == 2) {
    if (w.u.c + 1 < w.c1) {
      w.u.c++;
      return;
    }
    w.v += gridDim.x;
    if (w.v >= w.nv) { w.done = true; return; }
    walk_unit(p, w);
  } else if (p.order == 1) {
    if (++w.t >= w.t1) { w.done = true; return; }
    const TileCursor one{1, 0, 0, 0};
    cursor_add(p, w.u, one);
  } else {
    w.t += gridDim.x;
    if (w.t >= w.t1) { w.done = true; return; }
    w.u = cursor_of(p, w.t);
  }
}

__device__ __forceinline__ TileCoords coords_from(const RowPlan &p, const FieldDesc &f, const TileCursor &u,
                                                  const ColKey &ck)
{
  TileCoords t;
  t.c = u.c;
  t.jy = u.jy;
  t.jz = u.jz;
  t.r = u.r;
  t.jx0 = u.c * p.chunk;
  t.jx1 = t.jx0 + p.chunk < f.m[0] ? t.jx0 + p.chunk : f.m[0];
  t.skip = ck.skip;
  t.hi_x = ck.has_hi && u.c == p.nchunks - 1;
  return t;
}

// A slot is one piece of one staged row (NN*NP slots).  Slots are spread
// over the block's 256 threads: with more than 128 slots thread t takes
// slots t, t+256, ... (SPT of them) for every element of the tile; with
// fewer, KT = 256/(NN*NP) threads share a slot and thread t takes its
// elements k = t/(NN*NP), +KT, ... so that small tiles keep the block busy.
__host__ __device__ constexpr int slot_threads(int n)
{
  return n * n * pieces_per_row(n) <= 128 ? 256 / (n * n * pieces_per_row(n)) : 1;
}

// slot j of this thread (sl < 0: none) and its first element kq
template <int N, int SPT>
__device__ __forceinline__ void slot_of(int j, int &sl, int &kq)
{
  constexpr int S = N * N * pieces_per_row(N), KT = slot_threads(N);
  if constexpr (KT > 1) {
    static_assert(SPT == 1, "shared slots need one slot per thread");
    sl = (int)threadIdx.x % S;
    kq = (int)threadIdx.x / S;
    if (kq >= KT) sl = -1;
  } else {
    sl = (int)threadIdx.x + j * 256;
    kq = 0;
    if (sl >= S) sl = -1;
  }
}

// Stage one tile: per-slot column state (recomputed when the column changes),
// the row flags and x ends (one thread per row), and the cp.async copies.
// col holds at least SPT entries (SPTA >= SPT: a batched caller passes the
// largest array any n needs)
template <int N, int K, int SPT, int SPTA>
__device__ __forceinline__ void stage_tile(const FieldDesc &f, const RowPlan &p, const TileCursor &u, ColKey &ck,
                                           bool &have_col, SlotCol (&col)[SPTA], double *data, unsigned *rfl,
                                           double **lop, SlotCol *rinfo, int4 *tinfo)
{
  constexpr int NN = N * N, NP = pieces_per_row(N), PW = piece_doubles(N), RS = smem_row_stride(N);
  static_assert(SPTA >= SPT, "row source array too small");
  const bool newcol = !have_col || ck.r != u.r || ck.jy != u.jy || ck.jz != u.jz;
  if (newcol) {
    ck.r = u.r;
    ck.jy = u.jy;
    ck.jz = u.jz;
    ck.skip = (u.jy == f.m[1] && f.mode != kMessages && nbr_of(f, u.r, dir_index(0, 1, 0)) >= 0) ||
              (u.jz == f.m[2] && f.mode != kMessages && nbr_of(f, u.r, dir_index(0, 0, 1)) >= 0);
    ck.has_hi = f.mode == kMessages || nbr_of(f, u.r, dir_index(1, 0, 0)) < 0;
    have_col = true;
  }
  const TileCoords t = coords_from(p, f, u, ck);
  const int nk = t.skip ? 0 : t.jx1 - t.jx0;
  if (threadIdx.x == 0) *tinfo = make_int4(t.jx0, nk, t.hi_x ? 1 : 0, 0);
  double *buf = data, *locol = data + K * NN * RS, *hicol = locol + NN;
#pragma unroll
  for (int j = 0; j < SPT; j++) {
    int sl, kq;
    slot_of<N, SPT>(j, sl, kq);
    if (sl < 0) continue;
    const int r = sl / NP, pc = sl - (sl / NP) * NP;
    if (newcol) col[j] = slot_col(f, t, r);
    if (nk == 0) continue;
    const SlotCol &c = col[j];
    if (pc == 0 && kq == 0) {
      const double *lo, *hi;
      rfl[r] = row_ends(f, t, c, r, lo, hi);
      lop[r] = const_cast<double *>(lo);
      rinfo[r] = c;
      if (lo) cp_async(locol + r, lo, 1);
      if (hi) cp_async(hicol + r, hi, 1);
    }
    if (!(c.fl & kRowValid) || !piece_needed(N, c.fl, pc)) continue;
    constexpr int KT = slot_threads(N);
    const double *g = c.rd + (long)(t.jx0 + kq) * c.es + pc * PW;
    double *sp = buf + (kq * NN + r) * RS + pc * PW;
    for (int k = kq; k < nk; k += KT, g += KT * c.es, sp += KT * NN * RS) cp_async(sp, g, PW);
  }
  cp_commit();
}

}  // namespace tiledev

// shared memory layout, in doubles from a 16-byte aligned base: NS data
// stages, NS*N*N x-lower pointers, NS*N*N row flags (unsigned), NS tile
// infos (int4: jx0, nk, hi_x); every region starts on 16 bytes
template <int N, int K>
__host__ __device__ constexpr int tile_stage_size() { return K * N * N * smem_row_stride(N) + 2 * N * N; }
__host__ __device__ constexpr int round2(int d) { return (d + 1) & ~1; }
__host__ __device__ constexpr int lop_doubles(int n, int ns) { return round2(ns * n * n); }
__host__ __device__ constexpr int rfl_doubles(int n, int ns) { return (ns * n * n + 3) / 4 * 2; }
__host__ __device__ constexpr int rinfo_doubles(int n, int ns) { return ns * n * n * 2; }


namespace tiledev {

// Sum a staged tile: three dense passes when every row is present, else
// per-point groups with presence flags.
template <int N, int K>
__device__ __forceinline__ void sum_tile(double *buf, const unsigned *rfl, int nk, bool hx, bool regular)
{
  constexpr int NN = N * N, RS = smem_row_stride(N);
  double *locol = buf + K * NN * RS, *hicol = locol + NN;
  if (regular) {
    const int nx = (nk + (hx ? 1 : 0)) * NN;
    for (int i = threadIdx.x; i < nx; i += blockDim.x) xpass_at(N, nk, buf, locol, hicol, i / NN, i % NN);
    __syncthreads();
    const int span = nk * N + 1 + (hx ? 1 : 0);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nwarps = blockDim.x >> 5;
    for (int o = warp; o < N; o += nwarps)
      for (int c = lane; c < span; c += 32) yzpass_at(N, nk, 1, buf, locol, hicol, o, c);
    __syncthreads();
    for (int o = warp; o < N; o += nwarps)
      for (int c = lane; c < span; c += 32) yzpass_at(N, nk, 2, buf, locol, hicol, o, c);
  } else {
    const int groups = (int)tile_groups(N, nk, hx);
    for (int g = threadIdx.x; g < groups; g += blockDim.x) {
      int k, ix, iy, iz;
      group_point(N, nk, g, k, ix, iy, iz);
      tile_group_at(N, nk, rfl, buf, locol, hicol, k, ix, iy, iz);
    }
  }
}

// copy out: the changed rows, and the x-lower end where it is local
template <int N, int K, int SPT>
__device__ __forceinline__ void store_tile(const double *buf, const unsigned *rfl, double *const *lop,
                                           const SlotCol *rinfo, int jx0, int nk, bool hx)
{
  constexpr int NN = N * N, NP = pieces_per_row(N), PW = piece_doubles(N), RS = smem_row_stride(N);
  const double *locol = buf + K * NN * RS;
  if ((int)threadIdx.x < NN && (rfl[threadIdx.x] & kLoWritable)) *lop[threadIdx.x] = locol[threadIdx.x];
  constexpr int KT = slot_threads(N);
#pragma unroll
  for (int j = 0; j < SPT; j++) {
    int sl, kq;
    slot_of<N, SPT>(j, sl, kq);
    if (sl < 0) continue;
    const int r = sl / NP, pc = sl - (sl / NP) * NP;
    const SlotCol c = rinfo[r];
    if (!(c.fl & kRowWritable) || !piece_needed(N, c.fl, pc)) continue;
    double *g = const_cast<double *>(c.rd) + (long)(jx0 + kq) * c.es + pc * PW;
    const double *sp = buf + (kq * NN + r) * RS + pc * PW;
    for (int k = kq; k < nk; k += KT, g += KT * c.es, sp += KT * NN * RS) {
      const int len = slot_out_len(N, nk, hx, pc, k);
      if (PW == 2 && len == 2) *reinterpret_cast<double2 *>(g) = *reinterpret_cast<const double2 *>(sp);
      else if (len >= 1) *g = *sp;
    }
  }
}

}  // namespace tiledev

}  // namespace faces
