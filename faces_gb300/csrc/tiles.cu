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

struct TileState {
  long tile;
  int jx0, nk;
  int hi_x;
  int regular;
};

// issue the copies of tile `tile` into stage (meta, data); every thread works
// out the metadata of the rows it copies, so no barrier is needed here
template <int N, int K>
__device__ __forceinline__ void stage_in(const FieldDesc &f, const RowPlan &p, const TileCursor &cu, long tile,
                                         bool follow, const RowMeta *prev, TileState *ts, RowMeta *meta,
                                         double *data)
{
  constexpr int NN = N * N, NP = pieces_per_row(N), PW = piece_doubles(N), RS = smem_row_stride(N);
  const TileCoords t = coords_of(f, p, cu);
  const int nk = t.skip ? 0 : t.jx1 - t.jx0;
  if (threadIdx.x == 0) {
    ts->tile = tile;
    ts->jx0 = t.jx0;
    ts->nk = nk;
    ts->hi_x = (!t.skip && t.hi_x) ? 1 : 0;
    ts->regular = 0;
  }
  if (nk > 0) {
    double *buf = data, *locol = data + K * NN * RS, *hicol = locol + NN;
    for (int sl = threadIdx.x; sl < NN * NP; sl += blockDim.x) {
      const int r = sl / NP, pc = sl % NP;
      RowMeta m;
      tile_row_meta(f, t, follow, prev, r, m);
      if (pc == 0) {
        meta[r] = m;
        if (m.flags & kLoOk) cp_async(locol + r, m.lo, 1);
        if (m.flags & kHiOk) cp_async(hicol + r, m.hi, 1);
      }
      if (!(m.flags & kRowValid) || !piece_needed(N, m.flags, pc)) continue;
      Move mv;
      slot_move(N, m, r, pc, t.jx0, 0, buf, mv);
      const double *g = mv.g;
      double *sp = mv.s;
      for (int k = 0; k < nk; k++, g += m.es, sp += NN * RS) cp_async(sp, g, PW);
    }
  }
  cp_commit();
}

template <int N, int K>
__device__ __forceinline__ void stage_out(const TileState &ts, const RowMeta *meta, double *data)
{
  constexpr int NN = N * N, NP = pieces_per_row(N), PW = piece_doubles(N), RS = smem_row_stride(N);
  double *buf = data, *locol = data + K * NN * RS;
  for (int r = threadIdx.x; r < NN; r += blockDim.x) {
    const RowMeta &m = meta[r];
    if (m.flags & kLoWritable) *const_cast<double *>(m.lo) = locol[r];
  }
  for (int sl = threadIdx.x; sl < NN * NP; sl += blockDim.x) {
    const int r = sl / NP, pc = sl % NP;
    const RowMeta &m = meta[r];
    if (!(m.flags & kRowWritable) || !piece_needed(N, m.flags, pc)) continue;
    Move mv;
    slot_move(N, m, r, pc, ts.jx0, 0, buf, mv);
    double *g = const_cast<double *>(mv.g);
    const double *sp = mv.s;
    for (int k = 0; k < ts.nk; k++, g += m.es, sp += NN * RS) {
      const int len = slot_out_len(N, ts.nk, ts.hi_x != 0, pc, k);
      if (PW == 2 && len == 2) *reinterpret_cast<double2 *>(g) = *reinterpret_cast<const double2 *>(sp);
      else if (len >= 1) *g = *sp;
    }
  }
}

}  // namespace

// stage layout (doubles): NS data stages, then NS*N*N RowMeta, then NS TileState
template <int N, int K>
__host__ __device__ constexpr int tile_stage_size() { return K * N * N * smem_row_stride(N) + 2 * N * N; }

template <int N, int K, int NS>
__global__ void __launch_bounds__(256) tile_kernel(FieldDesc f, RowPlan p)
{
  constexpr int NN = N * N, RS = smem_row_stride(N);
  constexpr int stage = tile_stage_size<N, K>();
  extern __shared__ __align__(16) double sm[];
  RowMeta *meta_base = reinterpret_cast<RowMeta *>(sm + NS * stage);
  TileState *ts_base = reinterpret_cast<TileState *>(meta_base + NS * NN);

  // the block's tiles: a contiguous range (consecutive x-chunks of a
  // column: the row metadata carries over) or every gridDim.x-th tile
  long t0, t1, step;
  if (p.order == 1) {
    t0 = p.ntiles * blockIdx.x / gridDim.x;
    t1 = p.ntiles * (blockIdx.x + 1) / gridDim.x;
    step = 1;
  } else {
    t0 = blockIdx.x;
    t1 = p.ntiles;
    step = gridDim.x;
  }
  if (t0 >= t1) return;
  const TileCursor dstep = cursor_of(p, step);
  TileCursor nc = cursor_of(p, t0);  // next tile to stage
  long nt = t0;
  // prologue: the first NS-1 tiles in flight
#pragma unroll
  for (int j = 0; j < NS - 1; j++) {
    if (nt < t1) {
      // fresh metadata: the prologue has no barrier between its stages
      stage_in<N, K>(f, p, nc, nt, false, nullptr, ts_base + j, meta_base + j * NN, sm + j * stage);
      cursor_add(p, nc, dstep);
      nt += step;
    } else {
      cp_commit();
    }
  }
  // the loop reads row metadata and tile state that other threads wrote in
  // the prologue
  __syncthreads();
  int s = 0;
  for (long t = t0; t < t1; t += step) {
    cp_wait<NS - 2>();
    // tile t is staged; the block agrees whether it is regular
    const RowMeta *meta = meta_base + s * NN;
    bool ok = true;
    if ((int)threadIdx.x < NN) ok = row_regular(meta[threadIdx.x].flags, ts_base[s].hi_x != 0);
    const int regular = __syncthreads_and(ok);
    // the stage of the previous tile is free again: the next prefetch goes there
    const int sn = (s + NS - 1) % NS;
    if (nt < t1) {
      // contiguous order: nt-1 is staged in the stage before sn
      const bool follow = p.order == 1 && nc.c != 0;
      stage_in<N, K>(f, p, nc, nt, follow, meta_base + (sn - 1 + NS) % NS * NN, ts_base + sn,
                     meta_base + sn * NN, sm + sn * stage);
      cursor_add(p, nc, dstep);
      nt += step;
    } else {
      cp_commit();
    }
    const TileState cur = ts_base[s];
    double *buf = sm + s * stage, *locol = buf + K * NN * RS, *hicol = locol + NN;
    if (cur.nk > 0) {
      const bool hx = cur.hi_x != 0;
      if (regular) {
        const int nx = xpass_items(N, cur.nk, hx);
        for (int i = threadIdx.x; i < nx; i += blockDim.x) xpass_item(N, cur.nk, buf, locol, hicol, i);
        __syncthreads();
        const int ny = yzpass_items(N, cur.nk, hx);
        for (int i = threadIdx.x; i < ny; i += blockDim.x) yzpass_item(N, cur.nk, hx, 1, buf, locol, hicol, i);
        __syncthreads();
        for (int i = threadIdx.x; i < ny; i += blockDim.x) yzpass_item(N, cur.nk, hx, 2, buf, locol, hicol, i);
      } else {
        const int groups = (int)tile_groups(N, cur.nk, hx);
        for (int g = threadIdx.x; g < groups; g += blockDim.x) {
          int k, ix, iy, iz;
          group_point(N, cur.nk, g, k, ix, iy, iz);
          tile_group_at(N, cur.nk, meta, buf, locol, hicol, k, ix, iy, iz);
        }
      }
    }
    __syncthreads();
    if (cur.nk > 0) stage_out<N, K>(cur, meta, buf);
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
  return sizeof(double) * kTileStages * tile_stage_doubles(n, K) + kTileStages * sizeof(RowMeta) * n * n +
         kTileStages * sizeof(TileState);
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
