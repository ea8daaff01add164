// tiles.cu -- the shared-memory tile step (compute = true), sm_103a.
//
// Persistent CTAs walk the tiles of rows_setup.cuh.  Per tile: the staged
// rows arrive by cp.async (two stages: the next tile's copies are in flight
// while this one is summed), every owned shared point is summed once from
// shared memory by one thread (tile_ops.cuh), and the changed rows are stored
// back.  Global traffic is one read and one write of every row that holds a
// shared point; the FP64 adds are dense in every warp.
#include <cuda_runtime.h>

#include "geom.cuh"
#include "kernels.cuh"
#include "rows_setup.cuh"
#include "tile_ops.cuh"

namespace faces {

namespace {

__device__ __forceinline__ void cp_async(double *dst, const double *src, int len)
{
  const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
  if (len == 2)
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(d), "l"(src) : "memory");
  else
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(d), "l"(src) : "memory");
}

__device__ __forceinline__ void cp_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }

template <int W>
__device__ __forceinline__ void cp_wait() { asm volatile("cp.async.wait_group %0;" ::"n"(W) : "memory"); }

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

// Stage one tile: per-slot column state (recomputed when the column changes),
// the row flags and x ends (one thread per row), and the cp.async copies.
template <int N, int K, int SPT>
__device__ __forceinline__ void stage_tile(const FieldDesc &f, const RowPlan &p, const TileCursor &u, ColKey &ck,
                                           bool &have_col, SlotCol (&col)[SPT], double *data, unsigned *rfl,
                                           double **lop, SlotCol *rinfo, int4 *tinfo)
{
  constexpr int NN = N * N, NP = pieces_per_row(N), PW = piece_doubles(N), RS = smem_row_stride(N);
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
    const int sl = threadIdx.x + j * 256;
    if (sl >= NN * NP) continue;
    const int r = sl / NP, pc = sl - (sl / NP) * NP;
    if (newcol) col[j] = slot_col(f, t, r);
    if (nk == 0) continue;
    const SlotCol &c = col[j];
    if (pc == 0) {
      const double *lo, *hi;
      rfl[r] = row_ends(f, t, c, r, lo, hi);
      lop[r] = const_cast<double *>(lo);
      rinfo[r] = c;
      if (lo) cp_async(locol + r, lo, 1);
      if (hi) cp_async(hicol + r, hi, 1);
    }
    if (!(c.fl & kRowValid) || !piece_needed(N, c.fl, pc)) continue;
    const double *g = c.rd + (long)t.jx0 * c.es + pc * PW;
    double *sp = buf + r * RS + pc * PW;
    for (int k = 0; k < nk; k++, g += c.es, sp += NN * RS) cp_async(sp, g, PW);
  }
  cp_commit();
}

}  // namespace

// shared memory layout, in doubles from a 16-byte aligned base: NS data
// stages, NS*N*N x-lower pointers, NS*N*N row flags (unsigned), NS tile
// infos (int4: jx0, nk, hi_x); every region starts on 16 bytes
template <int N, int K>
__host__ __device__ constexpr int tile_stage_size() { return K * N * N * smem_row_stride(N) + 2 * N * N; }
__host__ __device__ constexpr int round2(int d) { return (d + 1) & ~1; }
__host__ __device__ constexpr int lop_doubles(int n, int ns) { return round2(ns * n * n); }
__host__ __device__ constexpr int rfl_doubles(int n, int ns) { return (ns * n * n + 3) / 4 * 2; }
__host__ __device__ constexpr int rinfo_doubles(int n, int ns) { return ns * n * n * 2; }

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
    double *buf = sm + s * stage, *locol = buf + K * NN * RS, *hicol = locol + NN;
    if (nk > 0) {
      if (regular) {
        const int nx = (nk + (hx ? 1 : 0)) * NN;
        for (int i = threadIdx.x; i < nx; i += blockDim.x) xpass_at(N, nk, buf, locol, hicol, i / NN, i % NN);
        __syncthreads();
        const int span = nk * N + 1 + (hx ? 1 : 0);
        const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
        for (int o = warp; o < N; o += 8)
          for (int c = lane; c < span; c += 32) yzpass_at(N, nk, 1, buf, locol, hicol, o, c);
        __syncthreads();
        for (int o = warp; o < N; o += 8)
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
    __syncthreads();
    if (nk > 0) {
      // copy out: the changed rows, and the x-lower end where it is local
      if ((int)threadIdx.x < NN && (rfl[threadIdx.x] & kLoWritable))
        *(lop_base + s * NN)[threadIdx.x] = locol[threadIdx.x];
#pragma unroll
      for (int j = 0; j < SPT; j++) {
        const int sl = threadIdx.x + j * 256;
        if (sl >= NN * NP) continue;
        const int r = sl / NP, pc = sl - (sl / NP) * NP;
        const SlotCol c = rinfo_base[s * NN + r];
        if (!(c.fl & kRowWritable) || !piece_needed(N, c.fl, pc)) continue;
        double *g = const_cast<double *>(c.rd) + (long)ti.x * c.es + pc * PW;
        const double *sp = buf + r * RS + pc * PW;
        for (int k = 0; k < nk; k++, g += c.es, sp += NN * RS) {
          const int len = slot_out_len(N, nk, hx, pc, k);
          if (PW == 2 && len == 2) *reinterpret_cast<double2 *>(g) = *reinterpret_cast<const double2 *>(sp);
          else if (len >= 1) *g = *sp;
        }
      }
    }
    s = (s + 1) % NS;
  }
}

bool tile_kernel_supported(int n) { return n >= 2 && n <= 12; }

// elements per tile: as many as fit a ~20 KB stage, at least 1 (three
// stages and three resident blocks per SM then fit in shared memory)
int tile_default_chunk(int n)
{
  const long per_elem = (long)n * n * smem_row_stride(n) * 8;
  long k = 20480 / per_elem;
  if (k < 1) k = 1;
  // the kernel is instantiated for these chunk sizes
  return k >= 8 ? 8 : k >= 4 ? 4 : k >= 2 ? 2 : 1;
}

constexpr int kTileStages = 3;

size_t tile_smem_bytes(int n, int chunk)
{
  const int K = tile_instance_k(chunk);
  // data stages, x-lower pointers, row flags, tile infos (see tile_kernel)
  return sizeof(double) * (kTileStages * tile_stage_doubles(n, K) + lop_doubles(n, kTileStages) +
                           rfl_doubles(n, kTileStages) + rinfo_doubles(n, kTileStages)) +
         sizeof(int4) * kTileStages;
}

template <int N, int K>
static cudaError_t launch_tiles_nk(const FieldDesc &f, const RowPlan &p, long grid, cudaStream_t s)
{
  static_assert(tile_stage_size<N, K>() * sizeof(double) % 16 == 0, "stage alignment");
  const size_t smem = tile_smem_bytes(N, K);
  // the attribute is set once per process (one device per process)
  static bool configured = false;
  if (!configured) {
    cudaError_t e =
        cudaFuncSetAttribute(tile_kernel<N, K, kTileStages>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    configured = true;
  }
  if (grid > p.ntiles) grid = p.ntiles;
  if (grid < 1) return cudaSuccess;
  tile_kernel<N, K, kTileStages><<<(unsigned)grid, 256, smem, s>>>(f, p);
  return cudaGetLastError();
}

template <int N>
static cudaError_t launch_tiles_n(const FieldDesc &f, const RowPlan &p, long grid, cudaStream_t s)
{
  if (p.chunk > 8) return cudaErrorInvalidValue;
  switch (tile_instance_k(p.chunk)) {
    case 1: return launch_tiles_nk<N, 1>(f, p, grid, s);
    case 2: return launch_tiles_nk<N, 2>(f, p, grid, s);
    case 4: return launch_tiles_nk<N, 4>(f, p, grid, s);
    case 8: return launch_tiles_nk<N, 8>(f, p, grid, s);
    default: return cudaErrorInvalidValue;
  }
}

cudaError_t launch_tiles(const FieldDesc &f, const RowPlan &p, long grid, cudaStream_t s)
{
  switch (f.n) {
    case 2: return launch_tiles_n<2>(f, p, grid, s);
    case 3: return launch_tiles_n<3>(f, p, grid, s);
    case 4: return launch_tiles_n<4>(f, p, grid, s);
    case 5: return launch_tiles_n<5>(f, p, grid, s);
    case 6: return launch_tiles_n<6>(f, p, grid, s);
    case 7: return launch_tiles_n<7>(f, p, grid, s);
    case 8: return launch_tiles_n<8>(f, p, grid, s);
    case 9: return launch_tiles_n<9>(f, p, grid, s);
    case 10: return launch_tiles_n<10>(f, p, grid, s);
    case 11: return launch_tiles_n<11>(f, p, grid, s);
    case 12: return launch_tiles_n<12>(f, p, grid, s);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace faces
