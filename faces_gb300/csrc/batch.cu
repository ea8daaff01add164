// batch.cu -- many independent fields, one persistent launch per share (the
// host side; the kernel is in batch_impl.cuh, its forms in batch_k*.cu).
//
// A batch holds fields of different shapes (rank grid, mx,my,mz, n).  One
// launch of batch_kernel advances every field by one share: the work list is
// every field's element columns cut into units of consecutive x-chunks,
// listed field by field and, inside a field, chunk group first, so the blocks
// running at one time hold neighbouring columns of one field.  Each block
// walks every gridDim.x-th unit through the same 3-stage cp.async pipeline as
// the single-field tile kernel, switching on each tile's n.  A CUDA graph of
// several launches replays the steps with one host call.  The plain form --
// one launch of the single-field kernel per field -- is kept for comparison.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdarg>
#include <cstdio>
#include <map>
#include <new>
#include <string>
#include <vector>

#include "../../include/faces_gb300.h"
#include "batch_kernel.h"
#include "ctx.h"
#include "geom.cuh"
#include "kernels.cuh"
#include "rows_setup.cuh"
#include "batch_impl.cuh"
#include "tile_ops.cuh"

void faces_internal_set_error(const char *msg);

namespace faces {


int batch_warp_chunk(int n) { return n >= kBatchMinN && n <= kBatchWarpMaxN ? bkw(n) : 0; }

void warp_split(long G, int nsmall, long nlarge, double small_pts, double large_pts, int boost, int run,
                int &wblocks, long &grid)
{
  long wb = 0;
  if (nsmall > 0) {
    wb = nlarge == 0 ? G
                     : std::max(1L, std::min(G - 1, (long)(G * small_pts * boost / (small_pts * boost + large_pts) + 0.5)));
    wb = std::min(wb, ((long)nsmall + 7) / 8);  // 8 warps a block
  }
  wblocks = (int)wb;
  // blocks of the block pipeline: the rest, no more than its runs
  const long runs = (nlarge + std::max(1, run) - 1) / std::max(1, run);
  grid = wb + std::max(nlarge > 0 ? 1L : 0L, std::min(G - wb, runs));
  if (grid < 1) grid = 1;
}

RowPlan batch_plan(const FieldDesc &f, int half, bool lean, bool warp)
{
  const int k = !batch_n_supported(f.n) ? 1 : (warp && lean && half != 1 && batch_warp_chunk(f.n)) ? bkw(f.n)
                : lean                                                                               ? bkl(f.n, half)
                                                                                                     : bk(f.n, half);
  RowPlan p = make_row_plan(f, k, 0);
  p.order = 2;
  p.unit_chunks = 1;
  return p;
}

int batch_blocks_per_sm(int half)
{
  return std::max(1, std::min(bblocks(half), (int)((228 * 1024) / (batch_smem_bytes(half) + 1024))));
}

cudaError_t batch_configure()
{
  cudaError_t e = batch_configure_00();
  if (e == cudaSuccess) e = batch_configure_20();
  if (e == cudaSuccess) e = batch_configure_10();
  if (e == cudaSuccess) e = batch_configure_11();
  if (e == cudaSuccess) e = batch_configure_12();
  return e;
}

int batch_mode(const BatchField *fields, size_t n)
{
  size_t lean = 0;
  for (size_t i = 0; i < n; i++) lean += fields[i].lean ? 1 : 0;
  return lean == 0 ? 0 : lean == n ? 1 : 2;
}

void append_units(std::vector<BatchUnit> &units, int field, const RowPlan &p, int unit_div)
{
  const long ncol = p.ntiles / p.nchunks;
  const int uc = std::max(1, (p.nchunks + unit_div - 1) / unit_div);
  for (int c0 = 0; c0 < p.nchunks; c0 += uc)
    for (long col = 0; col < ncol; col++) units.push_back({field, (int)col, c0, std::min(c0 + uc, p.nchunks)});
}

cudaError_t launch_batch(const BatchField *d_fields, const BatchUnit *d_units, int nunits, long grid, int run,
                         int mode, int half, cudaStream_t s, int nsmall, int wblocks)
{
  if (run < 1) run = 1;
  if (nunits <= 0 || grid <= 0) return cudaSuccess;
  if (half && mode != 1) return cudaErrorInvalidValue;  // half-length tiles: periodic step only
  // the warp form: mode 1, stage forms 0 and 2, some blocks left for the
  // other units unless there are none
  if (nsmall < 0 || nsmall > nunits || wblocks < 0 || wblocks > grid) return cudaErrorInvalidValue;
  if ((nsmall > 0) != (wblocks > 0) || (nsmall > 0 && (mode != 1 || half == 1))) return cudaErrorInvalidValue;
  if (nsmall < nunits && wblocks >= grid) return cudaErrorInvalidValue;
  if (mode == 1 && half == 2) return batch_launch_12(d_fields, d_units, nunits, grid, run, nsmall, wblocks, s);
  if (mode == 1 && half) return batch_launch_11(d_fields, d_units, nunits, grid, run, nsmall, wblocks, s);
  if (mode == 1) return batch_launch_10(d_fields, d_units, nunits, grid, run, nsmall, wblocks, s);
  if (mode == 2) return batch_launch_20(d_fields, d_units, nunits, grid, run, nsmall, wblocks, s);
  return batch_launch_00(d_fields, d_units, nunits, grid, run, nsmall, wblocks, s);
}

namespace {

int fail(int code, const char *fmt, ...)
{
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  faces_internal_set_error(buf);
  return code;
}

#define CUDA_TRY(call, what)                                                                      \
  do {                                                                                            \
    cudaError_t e_ = (call);                                                                      \
    if (e_ != cudaSuccess)                                                                        \
      return fail(e_ == cudaErrorMemoryAllocation ? FACES_ENOMEM : FACES_ECUDA, "%s: %s", what, \
                  cudaGetErrorString(e_));                                                        \
  } while (0)

}  // namespace
}  // namespace faces

using namespace faces;

struct faces_batch {
  std::vector<faces_ctx *> ctx;
  std::vector<double *> u;
  std::vector<char> fused;  // field runs in the batched kernel
  bool committed = false;
  BatchField *d_fields = nullptr;
  BatchUnit *d_units = nullptr;
  int nunits = 0;
  int run = 8;  // units a block takes in a row
  int mode = 0;      // batch_mode of the fused fields
  int half = 0;      // tile length form (mode 1 only): 0 default, 1 half (4 blocks/SM), 2 long (2 blocks/SM)
  int unit_div = 2;  // units are 1/unit_div of a column's chunks
  int per_sm = 3;
  int warp_n = kBatchWarpMaxN;  // fields with n up to this take the warp form (0: none)
  int boost = 2;                // warp blocks: boost x their share of the points
  int nsmall = 0;               // units of the warp form (listed first)
  int wblocks = 0;              // blocks that run them
  int sms = 0;
  long grid = 0;
  cudaStream_t capture = nullptr;
  std::map<long, cudaGraphExec_t> graphs;  // key: nshares*2 + compute
  std::vector<BatchField> h_fields;
};

namespace {

bool batch_eligible(const faces_ctx *c)
{
  // message strategies keep their own order of sums: one faces_share each
  return batch_n_supported(c->n) && !(c->flags & (FACES_MESSAGES | FACES_GATHER | FACES_ROWS | FACES_V6 | FACES_V6F | FACES_SEAMS));
}

void drop_graphs(faces_batch *b)
{
  for (auto &g : b->graphs) cudaGraphExecDestroy(g.second);
  b->graphs.clear();
}

// a batched field takes the warp form: every batched field on the periodic
// step (mode 1), not the half-length stages, n up to warp_n
bool warp_field(const faces_batch *b, const BatchField &bf)
{
  return b->mode == 1 && b->half != 1 && bf.lean && bf.f.n <= b->warp_n && batch_warp_chunk(bf.f.n) > 0;
}

// tile plans of every field for the current stage form and warp limit
int plan_fields(faces_batch *b)
{
  for (size_t i = 0; i < b->h_fields.size(); i++)
    b->h_fields[i].p = batch_plan(b->h_fields[i].f, b->half, b->h_fields[i].lean != 0, warp_field(b, b->h_fields[i]));
  if (!b->h_fields.empty())
    CUDA_TRY(cudaMemcpy(b->d_fields, b->h_fields.data(), sizeof(BatchField) * b->h_fields.size(),
                        cudaMemcpyHostToDevice),
             "faces_batch: field table upload");
  return FACES_OK;
}

int build_units(faces_batch *b)
{
  // fields in order of n, so that the blocks resident at one time mostly run
  // the code of one n; the warp form's fields (the smallest n) come first
  std::vector<size_t> order;
  for (size_t i = 0; i < b->h_fields.size(); i++)
    if (b->fused[i]) order.push_back(i);
  std::stable_sort(order.begin(), order.end(),
                   [&](size_t a, size_t c) { return b->h_fields[a].f.n < b->h_fields[c].f.n; });
  std::vector<BatchUnit> units;
  std::vector<BatchField> fused;
  double small_pts = 0, large_pts = 0;
  int nsmall = 0;
  for (size_t i : order) {
    const BatchField &bf = b->h_fields[i];
    const double pts = (double)bf.f.nranks * bf.f.m[0] * bf.f.m[1] * bf.f.m[2] * bf.f.n * bf.f.n * bf.f.n;
    fused.push_back(bf);
    if (warp_field(b, bf)) {
      append_units(units, (int)i, bf.p, 1);  // whole columns
      nsmall = (int)units.size();
      small_pts += pts;
    } else {
      append_units(units, (int)i, bf.p, b->unit_div);
      large_pts += pts;
    }
  }
  if (b->mode != 1 && b->half) return fail(FACES_EINVAL, "faces_batch: half-length tiles need all fields periodic");
  const long G = (long)b->sms * std::min(b->per_sm, batch_blocks_per_sm(b->half));
  b->nsmall = nsmall;
  warp_split(G, nsmall, (long)units.size() - nsmall, small_pts, large_pts, b->boost, b->run, b->wblocks, b->grid);
  cudaFree(b->d_units);
  b->d_units = nullptr;
  b->nunits = (int)units.size();
  if (!units.empty()) {
    CUDA_TRY(cudaMalloc(&b->d_units, sizeof(BatchUnit) * units.size()), "faces_batch: work list");
    CUDA_TRY(cudaMemcpy(b->d_units, units.data(), sizeof(BatchUnit) * units.size(), cudaMemcpyHostToDevice),
             "faces_batch: work list upload");
  }
  drop_graphs(b);
  return FACES_OK;
}

// stage form: full (0), half-length (1) or long (2) tiles
int set_half(faces_batch *b, int half)
{
  b->half = half;
  return plan_fields(b);
}

int launch_batched(faces_batch *b, cudaStream_t s)
{
  CUDA_TRY(launch_batch(b->d_fields, b->d_units, b->nunits, b->grid, b->run, b->mode, b->half, s, b->nsmall,
                        b->wblocks),
           "batch kernel launch");
  return FACES_OK;
}

int check_batch(const faces_batch *b, bool committed)
{
  if (!b) return fail(FACES_EINVAL, "null batch");
  if (committed && !b->committed) return fail(FACES_EINVAL, "batch not committed (faces_batch_commit)");
  if (!committed && b->committed) return fail(FACES_EINVAL, "batch already committed");
  return FACES_OK;
}

// one share of the fields the batched kernel does not take, one launch each
int share_others(faces_batch *b, int compute, bool all, void *stream)
{
  for (size_t i = 0; i < b->ctx.size(); i++)
    if (all || !b->fused[i] || !compute)
      if (int rc = faces_share(b->ctx[i], b->u[i], compute, stream)) return rc;
  return FACES_OK;
}

}  // namespace

extern "C" {

int faces_batch_create(faces_batch **out)
{
  if (!out) return fail(FACES_EINVAL, "null output pointer");
  faces_batch *b = new (std::nothrow) faces_batch();
  if (!b) return fail(FACES_ENOMEM, "host allocation failed");
  int dev = 0;
  cudaError_t e;
  if ((e = cudaGetDevice(&dev)) != cudaSuccess ||
      (e = cudaDeviceGetAttribute(&b->sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess) {
    delete b;
    return fail(FACES_ECUDA, "faces_batch_create: %s", cudaGetErrorString(e));
  }
  *out = b;
  return FACES_OK;
}

int faces_batch_add(faces_batch *b, double *u, int lx, int ly, int lz, int mx, int my, int mz, int n, unsigned flags,
                    int *field_id)
{
  if (int rc = check_batch(b, false)) return rc;
  if (!u || (reinterpret_cast<uintptr_t>(u) & 15u)) return fail(FACES_EALIGN, "field pointer null or not 16-byte aligned");
  faces_ctx *c = nullptr;
  if (int rc = faces_create(&c, lx, ly, lz, mx, my, mz, n, flags)) return rc;
  b->ctx.push_back(c);
  b->u.push_back(u);
  if (field_id) *field_id = (int)b->ctx.size() - 1;
  return FACES_OK;
}

int faces_batch_commit(faces_batch *b)
{
  if (int rc = check_batch(b, false)) return rc;
  const size_t nf = b->ctx.size();
  b->h_fields.resize(nf);
  b->fused.assign(nf, 0);
  for (size_t i = 0; i < nf; i++) {
    const faces_ctx *c = b->ctx[i];
    BatchField bf;
    bf.f = c->desc(b->u[i]);
    bf.lean = ptile_field(bf.f) && !(c->flags & FACES_GENERAL);
    bf.p = batch_plan(bf.f, 0, bf.lean != 0);
    b->h_fields[i] = bf;
    b->fused[i] = batch_eligible(c) ? 1 : 0;
  }
  std::vector<BatchField> fused;
  for (size_t i = 0; i < nf; i++)
    if (b->fused[i]) fused.push_back(b->h_fields[i]);
  b->mode = batch_mode(fused.data(), fused.size());
  if (nf) {
    CUDA_TRY(cudaMalloc(&b->d_fields, sizeof(BatchField) * nf), "faces_batch: field table");
    if (int rc = plan_fields(b)) return rc;
  }
  CUDA_TRY(batch_configure(), "faces_batch: shared memory attribute");
  b->per_sm = batch_blocks_per_sm(0);
  CUDA_TRY(cudaStreamCreateWithFlags(&b->capture, cudaStreamNonBlocking), "faces_batch: capture stream");
  b->committed = true;
  return build_units(b);
}

int faces_batch_share(faces_batch *b, int compute, void *stream)
{
  if (int rc = check_batch(b, true)) return rc;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (compute)
    if (int rc = launch_batched(b, s)) return rc;
  return share_others(b, compute, false, stream);
}

int faces_batch_share_n(faces_batch *b, int compute, int nshares, void *stream)
{
  if (int rc = check_batch(b, true)) return rc;
  if (nshares < 0) return fail(FACES_EINVAL, "nshares = %d must not be negative", nshares);
  if (nshares == 0) return FACES_OK;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const long key = (long)nshares * 2 + (compute ? 1 : 0);
  auto it = b->graphs.find(key);
  if (it == b->graphs.end()) {
    // capture nshares steps once; the graph replays them with one call
    cudaGraph_t g = nullptr;
    CUDA_TRY(cudaStreamBeginCapture(b->capture, cudaStreamCaptureModeThreadLocal), "faces_batch: begin capture");
    int rc = FACES_OK;
    for (int i = 0; i < nshares && rc == FACES_OK; i++) rc = faces_batch_share(b, compute, b->capture);
    const cudaError_t e = cudaStreamEndCapture(b->capture, &g);
    if (rc) {
      if (g) cudaGraphDestroy(g);
      return rc;
    }
    CUDA_TRY(e, "faces_batch: end capture");
    cudaGraphExec_t exec = nullptr;
    const cudaError_t e2 = cudaGraphInstantiate(&exec, g, 0);
    cudaGraphDestroy(g);
    CUDA_TRY(e2, "faces_batch: instantiate graph");
    it = b->graphs.emplace(key, exec).first;
  }
  CUDA_TRY(cudaGraphLaunch(it->second, s), "faces_batch: graph launch");
  return FACES_OK;
}

int faces_batch_share_each(faces_batch *b, int compute, void *stream)
{
  if (int rc = check_batch(b, true)) return rc;
  return share_others(b, compute, true, stream);
}

int faces_batch_tune(faces_batch *b, int unit_div, int blocks_per_sm, int half, int run)
{
  if (int rc = check_batch(b, true)) return rc;
  if (half > 0 && b->mode != 1) return fail(FACES_EINVAL, "half-length tiles need every batched field periodic");
  if (half > 2) return fail(FACES_EINVAL, "half = %d: 0, 1 or 2", half);
  if (half >= 0 && half != b->half)
    if (int rc = set_half(b, half)) return rc;
  if (unit_div > 0) b->unit_div = unit_div;
  if (blocks_per_sm > 0) b->per_sm = blocks_per_sm;
  if (run > 0) b->run = run;
  return build_units(b);
}

int faces_batch_autotune(faces_batch *b, int trials, void *stream)
{
  if (int rc = check_batch(b, true)) return rc;
  if (trials < 1) trials = 3;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  // candidates: tile length (full, or half when every field is periodic),
  // units per column, resident blocks per SM (the most that fit, one fewer)
  struct Cand {
    int half, div, per_sm, run;
  };
  std::vector<Cand> cands;
  const int divs[] = {1, 2, 4, 8, 64};
  const int runs[] = {1, 8};
  for (int h = 0; h < (b->mode == 1 ? 3 : 1); h++)
    for (int d : divs)
      for (int sm = batch_blocks_per_sm(h); sm >= std::max(1, batch_blocks_per_sm(h) - 1); sm--)
        for (int r : runs) cands.push_back({h, d, sm, r});
  cudaEvent_t e0, e1;
  CUDA_TRY(cudaEventCreate(&e0), "autotune: event");
  CUDA_TRY(cudaEventCreate(&e1), "autotune: event");
  float best = 1e30f;
  Cand pick{b->half, b->unit_div, b->per_sm, b->run};
  int applied = 0;  // shares the timed launches applied to each batched field
  int rc = FACES_OK;
  for (const Cand &c : cands) {
    if (c.half != b->half && (rc = set_half(b, c.half))) break;
    b->unit_div = c.div;
    b->per_sm = c.per_sm;
    b->run = c.run;
    if ((rc = build_units(b))) break;
    if (b->nunits == 0) break;
    if ((rc = launch_batched(b, s))) break;  // warm-up
    cudaEventRecord(e0, s);
    for (int t = 0; t < trials && rc == FACES_OK; t++) rc = launch_batched(b, s);
    cudaEventRecord(e1, s);
    applied += 1 + trials;
    if (rc) break;
    const cudaError_t e = cudaEventSynchronize(e1);
    if (e != cudaSuccess) {
      rc = fail(FACES_ECUDA, "autotune: synchronize: %s", cudaGetErrorString(e));
      break;
    }
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    if (ms < best) {
      best = ms;
      pick = c;
    }
  }
  if (rc == FACES_OK && pick.half != b->half) rc = set_half(b, pick.half);
  if (rc == FACES_OK) {
    b->unit_div = pick.div;
    b->per_sm = pick.per_sm;
    b->run = pick.run;
    rc = build_units(b);
  }
  // then the warp form: which small n take it, and its share of the blocks
  if (rc == FACES_OK && b->mode == 1 && b->half != 1) {
    int best_n = b->warp_n, best_boost = b->boost;
    best = 1e30f;
    const int wns[] = {0, 3, 4, kBatchWarpMaxN};
    const int boosts[] = {1, 2, 3, 4};
    for (int wn : wns)
      for (int bo : boosts) {
        if (rc != FACES_OK || (wn == 0 && bo > 1)) continue;
        b->warp_n = wn;
        b->boost = bo;
        if ((rc = plan_fields(b)) || (rc = build_units(b))) break;
        if ((rc = launch_batched(b, s))) break;
        cudaEventRecord(e0, s);
        for (int t = 0; t < trials && rc == FACES_OK; t++) rc = launch_batched(b, s);
        cudaEventRecord(e1, s);
        applied += 1 + trials;
        if (rc) break;
        const cudaError_t e = cudaEventSynchronize(e1);
        if (e != cudaSuccess) {
          rc = fail(FACES_ECUDA, "autotune: synchronize: %s", cudaGetErrorString(e));
          break;
        }
        float ms = 0;
        cudaEventElapsedTime(&ms, e0, e1);
        if (ms < best) {
          best = ms;
          best_n = wn;
          best_boost = bo;
        }
      }
    b->warp_n = best_n;
    b->boost = best_boost;
    if (rc == FACES_OK && (rc = plan_fields(b)) == FACES_OK) rc = build_units(b);
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (rc) return rc;
  return applied;
}

int faces_batch_tune_warp(faces_batch *b, int max_n, int boost)
{
  if (int rc = check_batch(b, true)) return rc;
  if (max_n > kBatchWarpMaxN) return fail(FACES_EINVAL, "max_n = %d: at most %d", max_n, kBatchWarpMaxN);
  if (max_n >= 0) b->warp_n = max_n;
  if (boost > 0) b->boost = boost;
  if (int rc = plan_fields(b)) return rc;
  return build_units(b);
}

int faces_batch_warp_info(const faces_batch *b, int *max_n, int *boost, int *warp_units, int *warp_blocks)
{
  if (!b) return fail(FACES_EINVAL, "null batch");
  if (max_n) *max_n = b->warp_n;
  if (boost) *boost = b->boost;
  if (warp_units) *warp_units = b->nsmall;
  if (warp_blocks) *warp_blocks = b->wblocks;
  return FACES_OK;
}

int faces_batch_info(const faces_batch *b, int *fields, int *fused_fields, int *units, int *unit_div, int *blocks,
                     int *half, int *run)
{
  if (!b) return fail(FACES_EINVAL, "null batch");
  int fu = 0;
  for (char c : b->fused) fu += c;
  if (fields) *fields = (int)b->ctx.size();
  if (fused_fields) *fused_fields = fu;
  if (units) *units = b->nunits;
  if (unit_div) *unit_div = b->unit_div;
  if (blocks) *blocks = (int)b->grid;
  if (half) *half = b->half;
  if (run) *run = b->run;
  return FACES_OK;
}

int faces_batch_destroy(faces_batch *b)
{
  if (!b) return FACES_OK;
  drop_graphs(b);
  if (b->capture) cudaStreamDestroy(b->capture);
  for (faces_ctx *c : b->ctx) faces_destroy(c);
  cudaFree(b->d_fields);
  cudaFree(b->d_units);
  delete b;
  return FACES_OK;
}

}  // extern "C"
