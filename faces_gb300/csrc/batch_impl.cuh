// batch_impl.cuh -- the batched kernel (templates on the kernel form).
// batch_k<MODE><H>.cu instantiate one form each, so that the build compiles
// them in parallel; batch.cu holds the host side.
#pragma once

#include <cuda_runtime.h>

#include "batch_kernel.h"
#include "geom.cuh"
#include "ptile_steps.cuh"
#include "rows_setup.cuh"
#include "tile_ops.cuh"
#include "tile_steps.cuh"

namespace faces {

using namespace tiledev;

namespace {

// elements per tile of the general step for each n, and the tiles that size
// the stage: as many as fit ~20 KB, a power of 2 (h = 1: half as many, so
// that stages are small enough for 4 resident blocks per SM; h = 2: as many
// as fit ~28 KB, 2 resident blocks per SM)
__host__ __device__ constexpr int pow2_floor(int k) { return k >= 32 ? 32 : k >= 16 ? 16 : k >= 8 ? 8 : k >= 4 ? 4 : k >= 2 ? 2 : 1; }
__host__ __device__ constexpr int bk(int n, int h)
{
  return h == 2 ? pow2_floor(28672 / (n * n * smem_row_stride(n) * 8))
         : h == 1 && tile_kmax(n) > 1 ? tile_kmax(n) / 2
                                       : tile_kmax(n);
}
__host__ __device__ constexpr int bblocks(int h) { return h == 2 ? 2 : h == 1 ? 4 : 3; }
__host__ __device__ constexpr int bspt(int n) { return (n * n * pieces_per_row(n) + 255) / 256; }

constexpr int kBatchStages = 3;
constexpr int kNNMax = kBatchMaxN * kBatchMaxN;

__host__ __device__ constexpr int cmax(int a, int b) { return a > b ? a : b; }
__host__ __device__ constexpr int stage_of(int n, int h) { return bk(n, h) * n * n * smem_row_stride(n) + 2 * n * n; }
__host__ __device__ constexpr int stage_max(int n, int h)
{
  return n < kBatchMinN ? 0 : cmax(stage_of(n, h), stage_max(n - 1, h));
}
__host__ __device__ constexpr int spt_max(int n) { return n < kBatchMinN ? 0 : cmax(bspt(n), spt_max(n - 1)); }

__host__ __device__ constexpr int stage_even(int h) { return (stage_max(kBatchMaxN, h) + 1) & ~1; }
template <int H>
constexpr int kStage = stage_even(H);
constexpr int kSptMax = spt_max(kBatchMaxN);

// elements per tile of the periodic step: as many as the stage holds, at
// most 32.  The stage is sized by the n whose power-of-2 tile needs the most
// room (n = 8 at h = 0), so the other n get longer tiles than bk (at h = 0:
// n = 4 takes 27 elements, 5: 17, 6: 12, 7: 5, 9: 3).  The periodic step's
// loops take any tile length.
__host__ __device__ constexpr int bkl(int n, int h)
{
  return (stage_even(h) - 2 * n * n) / (n * n * smem_row_stride(n)) > 32
             ? 32
             : (stage_even(h) - 2 * n * n) / (n * n * smem_row_stride(n));
}
__host__ __device__ constexpr bool bkl_fits(int n, int h)
{
  return n > kBatchMaxN || (bkl(n, h) >= bk(n, h) && bkl(n, h) * n * n * smem_row_stride(n) + 2 * n * n <= stage_even(h) &&
                            bkl_fits(n + 1, h));
}
static_assert(bkl_fits(kBatchMinN, 0) && bkl_fits(kBatchMinN, 1) && bkl_fits(kBatchMinN, 2),
              "periodic-step tiles fit the stage");

// The warp form for small n (periodic step, stage forms h = 0 and 2): each
// of a block's 8 warps stages, sums and stores its own tiles in one eighth
// of the data stages (kWarpStage doubles), without block barriers; tiles of
// up to 32 elements that fill that share (n = 2: 32, 3: 18, 4: 10, 5: 6).
constexpr int kWarpStage = (kBatchStages * kStage<0> / 8) & ~1;
__host__ __device__ constexpr int bkw(int n)
{
  return (kWarpStage - 2 * n * n) / (n * n * smem_row_stride(n)) > 32
             ? 32
             : (kWarpStage - 2 * n * n) / (n * n * smem_row_stride(n));
}
static_assert(kStage<2> >= kStage<0>, "the warp form fits the long stages too");
static_assert(bkw(kBatchWarpMaxN) >= 1, "warp tiles hold an element");

// shared memory: data stages, then per-stage row arrays sized for n = 10
constexpr long batch_smem_bytes(int h)
{
  return sizeof(double) * (long)kBatchStages * (h == 2 ? kStage<2> : h ? kStage<1> : kStage<0>) + sizeof(double *) * (long)kBatchStages * kNNMax +
         sizeof(SlotCol) * (long)kBatchStages * kNNMax + sizeof(unsigned) * (long)kBatchStages * kNNMax +
         sizeof(int4) * kBatchStages + sizeof(PMeta) * kBatchStages + 2 * sizeof(BatchField);
}

struct BWalk {
  int u, u_end, run_index, c, c1, field;  // unit, end and index of the current run of units
  TileCursor cur;
  bool done;
};

__device__ __forceinline__ void bwalk_unit(const BatchField *fields, const BatchUnit *units, BWalk &w)
{
  const BatchUnit un = units[w.u];
  w.field = un.field;
  w.c = un.c0;
  w.c1 = un.c1;
  const RowPlan &p = fields[un.field].p;
  w.cur = cursor_of(p, (long)un.column * p.nchunks + un.c0);
}

// Blocks take runs of `run` consecutive units: block b the runs b, b + grid,
// b + 2 grid, ...  Consecutive tiles of a block then mostly belong to one
// field (its description stays in shared memory), and the blocks running at
// one time cover a narrow window of the work list (fields in order of n: one
// n's code).
__device__ __forceinline__ bool bwalk_run(int run, int nunits, int r, BWalk &w)
{
  w.run_index = r;
  w.u = r * run;
  w.u_end = min(w.u + run, nunits);
  return w.u < nunits;
}

__device__ __forceinline__ void bwalk_next(const BatchField *fields, const BatchUnit *units, int nunits, int run,
                                           int stride, BWalk &w)
{
  if (w.c + 1 < w.c1) {
    w.c++;
    w.cur.c++;
    return;
  }
  if (++w.u >= w.u_end) {
    if (!bwalk_run(run, nunits, w.run_index + stride, w)) {
      w.done = true;
      return;
    }
  }
  bwalk_unit(fields, units, w);
}

struct Smem {
  double *data;
  double **lop;
  SlotCol *rinfo;
  unsigned *rfl;
  int4 *tinfo;
  PMeta *meta;
  BatchField *field;  // two slots: the block's copies of the fields it stages
};

template <int H>
__device__ __forceinline__ Smem smem_layout(double *sm)
{
  static_assert(kStage<H> % 2 == 0, "stages keep 16-byte alignment");
  static_assert((kBatchStages * kNNMax * sizeof(unsigned)) % 16 == 0, "tile infos stay 16-byte aligned");
  Smem m;
  m.data = sm;
  m.lop = reinterpret_cast<double **>(sm + (long)kBatchStages * kStage<H>);
  m.rinfo = reinterpret_cast<SlotCol *>(m.lop + kBatchStages * kNNMax);
  m.rfl = reinterpret_cast<unsigned *>(m.rinfo + kBatchStages * kNNMax);
  m.tinfo = reinterpret_cast<int4 *>(m.rfl + kBatchStages * kNNMax);
  m.meta = reinterpret_cast<PMeta *>(m.tinfo + kBatchStages);
  m.field = reinterpret_cast<BatchField *>(m.meta + kBatchStages);
  return m;
}

// MODE: 0 every field takes the general step, 1 every field the periodic
// step, 2 each field its own
template <int N, int MODE, int H>
__device__ __forceinline__ void bstage(const BatchField &bf, const TileCursor &u, ColKey &ck, bool &have_col,
                                       SlotCol (&col)[kSptMax], const Smem &m, int st)
{
  if (MODE == 1 || (MODE == 2 && bf.lean))
    ptile::pstage<N, bkl(N, H)>(bf.f, bf.p, u, m.data + (long)st * kStage<H>, m.meta + st, m.tinfo + st,
                                threadIdx.x);
  else
    stage_tile<N, bk(N, H), bspt(N)>(bf.f, bf.p, u, ck, have_col, col, m.data + (long)st * kStage<H>,
                                  m.rfl + st * kNNMax, m.lop + st * kNNMax, m.rinfo + st * kNNMax, m.tinfo + st);
}

constexpr int kFieldWords = (int)(sizeof(BatchField) / 8);

// copy field `field` into a shared slot, with a barrier on each side (the
// prologue only: in the main loop the copy of the next tile's field is
// loaded early and stored into the other slot before the loop's barrier).
// Block-uniform: every thread sees the same field.
__device__ __forceinline__ void load_field(const BatchField *fields, int field, BatchField *slot, int &cached)
{
  if (field == cached) return;
  static_assert(sizeof(BatchField) % 8 == 0, "field table entries are whole words");
  const long long *src = reinterpret_cast<const long long *>(fields + field);
  long long *dst = reinterpret_cast<long long *>(slot);
  __syncthreads();
  for (int i = threadIdx.x; i < kFieldWords; i += blockDim.x) dst[i] = src[i];
  __syncthreads();
  cached = field;
}

// stage tile u of field `field` (its copy: bf) into stage st; the tile
// info's z holds hi_x | lean << 1 | n << 2 and w the field
template <int MODE, int H>
__device__ __forceinline__ void bstage_any(int field, const BatchField &bf, const TileCursor &u, ColKey &ck,
                                           bool &have_col, SlotCol (&col)[kSptMax], const Smem &m, int st)
{
  switch (bf.f.n) {
#define FACES_BSTAGE(NV) \
  case NV: bstage<NV, MODE, H>(bf, u, ck, have_col, col, m, st); break;
    FACES_BSTAGE(2) FACES_BSTAGE(3) FACES_BSTAGE(4) FACES_BSTAGE(5) FACES_BSTAGE(6) FACES_BSTAGE(7) FACES_BSTAGE(8)
    FACES_BSTAGE(9) FACES_BSTAGE(10)
#undef FACES_BSTAGE
    default:
      if (threadIdx.x == 0) m.tinfo[st] = make_int4(0, 0, 0, 0);
      cp_commit();
      break;
  }
  if (threadIdx.x == 0) {
    int4 ti = m.tinfo[st];
    ti.z = (ti.z & 1) | ((MODE == 1 || (MODE == 2 && bf.lean)) ? 2 : 0) | (bf.f.n << 2);
    ti.w = field;
    m.tinfo[st] = ti;
  }
}

// one tile of the warp form: stage, wait, x pairs, y/z pairs, by one warp
template <int N>
__device__ __forceinline__ void warp_tile(const BatchField *bf, const TileCursor &u, double *buf, PMeta *meta,
                                          int4 *tinfo, int lane)
{
  constexpr int KW = bkw(N);
  ptile::pstage<N, KW, 32>(bf->f, bf->p, u, buf, meta, tinfo, lane);
  cp_wait<0>();
  __syncwarp();
  const int nk = tinfo->y;
  ptile::pxpass<N, KW, 32>(meta->u, buf, meta, nk, lane);
  __syncwarp();
  ptile::pyzpass<N, KW, 32>(meta->u, buf, meta, nk, lane);
  __syncwarp();
}

// Units [0, nsmall) are small-n fields' (periodic step, tiles of bkw(n)
// elements): blocks [0, wblocks) take them, warp by warp (unit q: warp
// q % (8 * wblocks) of the warp blocks).  The other blocks walk units
// [nsmall, nunits) through the block pipeline.  MODE 1 only.
template <int MODE, int H>
__device__ __forceinline__ void warp_units(const BatchField *fields, const BatchUnit *units, int nsmall, int wblocks,
                                           const Smem &m)
{
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  double *buf = m.data + (long)warp * kWarpStage;
  // the per-stage row arrays of the general step are unused here: they hold
  // each warp's tile record
  PMeta *meta = reinterpret_cast<PMeta *>(m.lop) + warp;
  int4 *tinfo = reinterpret_cast<int4 *>(reinterpret_cast<PMeta *>(m.lop) + 8) + warp;
  for (int q = blockIdx.x * 8 + warp; q < nsmall; q += wblocks * 8) {
    const BatchUnit un = units[q];
    const BatchField *bf = fields + un.field;
    const int n = bf->f.n, nchunks = bf->p.nchunks;
    TileCursor u = cursor_of(bf->p, (long)un.column * nchunks + un.c0);
    for (int c = un.c0; c < un.c1; c++, u.c++) {
      switch (n) {
        case 2: warp_tile<2>(bf, u, buf, meta, tinfo, lane); break;
        case 3: warp_tile<3>(bf, u, buf, meta, tinfo, lane); break;
        case 4: warp_tile<4>(bf, u, buf, meta, tinfo, lane); break;
        case 5: warp_tile<5>(bf, u, buf, meta, tinfo, lane); break;
        default: break;
      }
    }
  }
}

template <int MODE, int H>
__global__ void __launch_bounds__(256, bblocks(H))
    batch_kernel(const BatchField *fields, const BatchUnit *units_all, int nunits_all, int run, int nsmall,
                 int wblocks)
{
  extern __shared__ __align__(16) double sm[];
  const Smem m = smem_layout<H>(sm);
  if constexpr (MODE == 1 && H != 1) {
    if ((int)blockIdx.x < wblocks) {
      warp_units<MODE, H>(fields, units_all, nsmall, wblocks, m);
      return;
    }
  }
  // the block pipeline: units [nsmall, nunits_all), blocks [wblocks, grid)
  const BatchUnit *units = units_all + nsmall;
  const int nunits = nunits_all - nsmall, stride = (int)gridDim.x - wblocks;
  BWalk nw;  // next tile to stage
  nw.done = !bwalk_run(run, nunits, (int)blockIdx.x - wblocks, nw);
  if (nw.done) return;
  bwalk_unit(fields, units, nw);
  ColKey ck{};
  bool have_col = false;
  int last_field = -1;
  // field slots: the next tile to stage takes slot `cur` (holding field
  // cached_cur); the other slot holds cached_oth
  int cur = 0, cached_cur = -1, cached_oth = -1;
  SlotCol col[kSptMax];
  int inflight = 0;
#pragma unroll
  for (int j = 0; j < kBatchStages - 1; j++) {
    if (!nw.done) {
      if (nw.field != last_field) { have_col = false; last_field = nw.field; }
      load_field(fields, nw.field, m.field + cur, cached_cur);
      bstage_any<MODE, H>(nw.field, m.field[cur], nw.cur, ck, have_col, col, m, j);
      bwalk_next(fields, units, nunits, run, stride, nw);
      inflight++;
    } else {
      cp_commit();
    }
  }
  if (!nw.done) load_field(fields, nw.field, m.field + cur, cached_cur);
  __syncthreads();
  int s = 0;
  for (; inflight > 0; inflight--) {
    cp_wait<kBatchStages - 2>();
    const unsigned *rfl = m.rfl + s * kNNMax;
    const int4 ti = m.tinfo[s];
    const int nk = ti.y, n = ti.z >> 2;
    const bool hx = (ti.z & 1) != 0, lean = MODE == 1 || (MODE == 2 && (ti.z & 2) != 0);
    bool ok = true;
    if (!lean && (int)threadIdx.x < n * n) ok = row_regular(rfl[threadIdx.x], hx);
    const int regular = __syncthreads_and(ok);
    const int sn = (s + kBatchStages - 1) % kBatchStages;
    if (!nw.done) {
      if (nw.field != last_field) { have_col = false; last_field = nw.field; }
      bstage_any<MODE, H>(nw.field, m.field[cur], nw.cur, ck, have_col, col, m, sn);
      bwalk_next(fields, units, nunits, run, stride, nw);
      inflight++;
      // the field of the tile staged next: already in a slot, or copied now
      // into the other slot, which nobody reads in this iteration (its last
      // readers staged before this iteration's barrier; the next iteration's
      // barrier publishes the copy)
      if (!nw.done && nw.field != cached_cur) {
        if (nw.field != cached_oth) {
          if ((int)threadIdx.x < kFieldWords)
            reinterpret_cast<long long *>(m.field + (cur ^ 1))[threadIdx.x] =
                reinterpret_cast<const long long *>(fields + nw.field)[threadIdx.x];
          cached_oth = nw.field;
        }
        const int was = cached_cur;
        cached_cur = cached_oth;
        cached_oth = was;
        cur ^= 1;
      }
    } else {
      cp_commit();
    }
    double *buf = m.data + (long)s * kStage<H>;
    double *const fu = m.meta[s].u;  // the field of this tile (periodic step)
    // periodic step: x pairs, barrier, y/z pairs (each storing its finals);
    // general step: sums (with their own barriers), barrier, store
    if (nk > 0) {
      switch (n) {
#define FACES_BSUM(NV)                                                       \
  case NV:                                                                   \
    if (lean) ptile::pxpass<NV, bkl(NV, H)>(fu, buf, m.meta + s, nk, threadIdx.x);            \
    else sum_tile<NV, bk(NV, H)>(buf, rfl, nk, hx, regular != 0);               \
    break;
        FACES_BSUM(2) FACES_BSUM(3) FACES_BSUM(4) FACES_BSUM(5) FACES_BSUM(6) FACES_BSUM(7) FACES_BSUM(8)
        FACES_BSUM(9) FACES_BSUM(10)
#undef FACES_BSUM
        default: break;
      }
    }
    __syncthreads();
    if (nk > 0) {
      switch (n) {
#define FACES_BSTORE(NV)                                                                                  \
  case NV:                                                                                                 \
    if (lean)                                                                                              \
      ptile::pyzpass<NV, bkl(NV, H)>(fu, buf, m.meta + s, nk, threadIdx.x);                                \
    else                                                                                                   \
      store_tile<NV, bk(NV, H), bspt(NV)>(buf, rfl, m.lop + s * kNNMax, m.rinfo + s * kNNMax, ti.x, nk, hx); \
    break;
        FACES_BSTORE(2) FACES_BSTORE(3) FACES_BSTORE(4) FACES_BSTORE(5) FACES_BSTORE(6) FACES_BSTORE(7)
        FACES_BSTORE(8) FACES_BSTORE(9) FACES_BSTORE(10)
#undef FACES_BSTORE
        default: break;
      }
    }
    s = (s + 1) % kBatchStages;
  }
}

}  // namespace

template <int MODE, int H>
cudaError_t batch_configure_t()
{
  return cudaFuncSetAttribute(batch_kernel<MODE, H>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)batch_smem_bytes(H));
}

template <int MODE, int H>
cudaError_t batch_launch_t(const BatchField *fields, const BatchUnit *units, int nunits, long grid, int run,
                           int nsmall, int wblocks, cudaStream_t s)
{
  batch_kernel<MODE, H><<<(unsigned)grid, 256, batch_smem_bytes(H), s>>>(fields, units, nunits, run, nsmall, wblocks);
  return cudaGetLastError();
}

}  // namespace faces
