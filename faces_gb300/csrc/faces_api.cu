// faces_api.cu -- the C ABI of include/faces_gb300.h.
//
// Host side of the reference's Faces class (gpu/v-26-messages/Faces.cc:10-103)
// for lx*ly*lz virtual ranks at once: neighbour tables, direction-keyed
// message buffers, launch of the sm_103a kernels in kernels.cu.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdarg>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "../../include/faces_gb300.h"
#include "pack_steps.cuh"
#include "geom.cuh"
#include "kernels.cuh"
#include "tables.h"
#include "ctx.h"
#include "tile_ops.cuh"

using namespace faces;

namespace {

thread_local std::string g_err;

int fail(int code, const char *fmt, ...)
{
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_err = buf;
  return code;
}

int cuda_fail(cudaError_t e, const char *what)
{
  return fail(e == cudaErrorMemoryAllocation ? FACES_ENOMEM : FACES_ECUDA, "%s: %s (%s)", what,
              cudaGetErrorString(e), cudaGetErrorName(e));
}

#define CUDA_TRY(call, what)                  \
  do {                                        \
    cudaError_t e_ = (call);                  \
    if (e_ != cudaSuccess) return cuda_fail(e_, what); \
  } while (0)

bool aligned16(const void *p) { return (reinterpret_cast<uintptr_t>(p) & 15u) == 0; }

}  // namespace

// error text for faces_last_error() from the other translation units
void faces_internal_set_error(const char *msg) { g_err = msg; }

namespace {

// default x-chunk: whole rows when that already fills the GPU, else split
// rows until about 150k threads are resident
int default_chunk(const faces_ctx &c)
{
  const bool virt = (c.flags & FACES_MESSAGES) || !(c.flags & FACES_PERIODIC);
  const long rows = (long)c.nranks * (c.m[1] + virt) * (c.m[2] + virt);
  const int P = c.n <= 2 ? 2 : c.n <= 4 ? 4 : c.n <= 8 ? 8 : 16;
  const long tt = ((P * c.n + 31) / 32) * 32;
  const long want = 152L * 1024;
  long nch = (want + rows * tt - 1) / (rows * tt);
  if (nch < 1) nch = 1;
  if (nch > c.m[0]) nch = c.m[0];
  return (int)((c.m[0] + nch - 1) / nch);
}

// v-26 message mode on a field with no neighbour rank (one non-periodic
// rank) has no message to pack or read: its share is the direct step's
bool no_messages(const faces_ctx &c) { return (c.flags & FACES_MESSAGES) && c.msg_total == 0; }

// the seam kernel runs this share: forced, the default, or chosen by
// autotune (variant 3)
bool seam_step(const faces_ctx &c)
{
  return (c.variant == 3 || (c.flags & FACES_SEAMS)) && seam_kernel_supported(c.n) &&
         !(c.flags & (FACES_V6 | FACES_V6F | FACES_GATHER)) && (!(c.flags & FACES_MESSAGES) || no_messages(c));
}

// message mode with FACES_PACK_FUSED: the pack runs in the message-mode
// tile kernel's prologue (one launch per share) when that kernel runs
bool pack_in_tiles(const faces_ctx &c, int compute)
{
  const bool general = (c.flags & FACES_GENERAL) || c.variant == 1;
  return (c.flags & FACES_MESSAGES) && (c.flags & FACES_PACK_FUSED) && !(c.flags & (FACES_GATHER | FACES_ROWS)) &&
         compute && !general && c.variant == 0 && c.tplan.order != 3 && tile_kernel_supported(c.n);
}

// The default kernel: the seam kernel for direct-mode fields with n >= 11,
// where it moves more than the tile step (95x94x93 n = 12: 3.71 ms per share
// open against 4.90, 3.85 periodic against 4.34; 15x14x13 n = 12: 0.024 against 0.029;
// 40^3 n = 11 periodic: 0.259 against 0.276; the tile step wins at n = 10:
// 48^3 0.313 against 0.353) and the tile step does not reach past n = 12;
// else the tile step.
int default_variant(const faces_ctx &c)
{
  return c.n >= 11 && seam_kernel_supported(c.n) &&
                 !(c.flags & (FACES_V6 | FACES_V6F | FACES_GATHER | FACES_ROWS | FACES_GENERAL)) &&
                 (!(c.flags & FACES_MESSAGES) || no_messages(c))
             ? 3
             : 0;
}

void replan(faces_ctx &c)
{
  const FieldDesc f = c.desc(nullptr);
  c.plan = make_row_plan(f, c.chunk > 0 ? c.chunk : default_chunk(c), c.tpb);
  if (seam_step(c)) {
    // resident blocks per SM from the kernel's occupancy (or the width asked for)
    const int fit = seam_blocks_per_sm(c.n);
    // order 1: the lean form, 0: the chunked form; by default the lean form
    // where it gives the GPU four waves of threads (measured: 95x94x93 n = 12
    // 3.71 ms lean, 4.82 chunked; 15x14x13 n = 12 0.025 lean, 0.023 chunked)
    const long lean_threads = (long)c.nranks * c.m[0] * c.m[1] * c.m[2] * (c.n > 2 ? (c.n - 2) * (c.n - 2) : 1);
    const bool lean = c.order == 1 || (c.order < 0 && lean_threads >= 4L * c.sms * 6 * 256);
    c.splan = make_seam_plan(f, c.chunk, (long)c.sms * (c.tpb > 0 && c.tpb < fit ? c.tpb : fit), lean);
  }
  if (tile_kernel_supported(c.n)) {
    // the tile kernel is built for 1, 2, 4, ... tile_kinst_max(n) elements
    // per tile: a requested chunk rounds down to one of them
    const bool general = (c.flags & FACES_GENERAL) || c.variant == 1;
    const TileForm form = tile_form(f, general);
    int k = c.chunk > 0 ? c.chunk : tile_default_chunk(c.n, form);
    int k2 = 1;
    while (k2 * 2 <= k && k2 * 2 <= tile_kinst_max(c.n)) k2 *= 2;
    k = k2;
    // the form's shared memory at most 110 KB (two blocks per SM)
    while (k > 1 && tile_form_smem_bytes(c.n, k, form) > 110 * 1024) k /= 2;
    // a default longer than the ~20 KB stage only where every block of two
    // per SM still gets four tiles
    if (c.chunk <= 0) {
      const bool virt = (c.flags & FACES_MESSAGES) || !(c.flags & FACES_PERIODIC);
      const long cols = (long)c.nranks * (c.m[1] + virt) * (c.m[2] + virt);
      while (k > tile_kmax(c.n) && cols * ((c.m[0] + k - 1) / k) < 4L * 2 * c.sms) k /= 2;
    }
    c.tplan = make_row_plan(f, k, 0);
    // order 3 (warp tiles) applies to the periodic step only; elsewhere it
    // means the default
    c.tplan.order = c.order >= 0 && c.order % 16 != 3 ? (c.order % 16) : 2;
    // order 2 units: chunks per unit (tuning value order = 2 + 16*u), default
    // half a column
    const int uc = c.order >= 16 ? c.order / 16 : (c.tplan.nchunks + 1) / 2;
    c.tplan.unit_chunks = uc < 1 ? 1 : uc;
    // resident blocks per SM: shared memory (228 KB per SM, 1 KB reserved
    // per block) and 2048 threads of 256-thread blocks
    const bool periodic_step = (c.flags & FACES_PERIODIC) && !(c.flags & (FACES_MESSAGES | FACES_GENERAL));
    const int fit = tile_blocks_per_sm(c.n, k, form);
    const int per_sm = c.tpb > 0 ? (c.tpb < fit ? c.tpb : fit) : fit;
    c.tgrid = (long)c.sms * (per_sm < 1 ? 1 : per_sm);
    if (periodic_step && c.order >= 0 && c.order % 16 == 3) {
      // warp tiles: one warp per tile of tile_kwarp(n) elements
      c.tplan = make_row_plan(f, tile_kwarp(c.n), 0);
      c.tplan.order = 3;
      c.tplan.unit_chunks = 1;
      const int wfit = wtile_blocks_per_sm(c.n);
      c.tgrid = (long)c.sms * (c.tpb > 0 && c.tpb < wfit ? c.tpb : wfit);
    }
  }
}

int check_ctx(const faces_ctx *c)
{
  if (!c) return fail(FACES_EINVAL, "null context");
  return FACES_OK;
}

int check_field(const double *u)
{
  if (!u) return fail(FACES_EINVAL, "null field pointer");
  if (!aligned16(u)) return fail(FACES_EALIGN, "field pointer %p is not 16-byte aligned", (const void *)u);
  return FACES_OK;
}

}  // namespace

extern "C" {

const char *faces_last_error(void) { return g_err.c_str(); }

int faces_create(faces_ctx **out, int lx, int ly, int lz, int mx, int my, int mz, int n, unsigned flags)
{
  if (!out) return fail(FACES_EINVAL, "null output pointer");
  *out = nullptr;
  if (lx < 1 || ly < 1 || lz < 1) return fail(FACES_EINVAL, "rank grid %d x %d x %d must be positive", lx, ly, lz);
  if (mx < 1 || my < 1 || mz < 1) return fail(FACES_EINVAL, "element grid %d x %d x %d must be positive", mx, my, mz);
  if (n < 2) return fail(FACES_EINVAL, "element size n = %d: n must be at least 2", n);
  if (flags & ~(FACES_PERIODIC | FACES_MESSAGES | FACES_GATHER | FACES_ROWS | FACES_GENERAL | FACES_V6 | FACES_V6F |
                FACES_SEAMS | FACES_PACK_FUSED))
    return fail(FACES_EINVAL, "unknown flags 0x%x", flags);
  if ((flags & FACES_SEAMS) && (flags & (FACES_MESSAGES | FACES_V6 | FACES_V6F)))
    return fail(FACES_EINVAL, "FACES_SEAMS sums every copy in place: not with a message strategy");
  if (((flags & FACES_V6) != 0) + ((flags & FACES_V6F) != 0) + ((flags & FACES_MESSAGES) != 0) > 1)
    return fail(FACES_EINVAL, "FACES_V6, FACES_V6F and FACES_MESSAGES are message strategies: choose one");
  const long nranks = (long)lx * ly * lz;
  if (nranks > 65535 / 27) return fail(FACES_EINVAL, "%ld ranks: at most %d virtual ranks", nranks, 65535 / 27);
  faces_ctx *c = new (std::nothrow) faces_ctx();
  if (!c) return fail(FACES_ENOMEM, "host allocation failed");
  c->L[0] = lx; c->L[1] = ly; c->L[2] = lz;
  c->m[0] = mx; c->m[1] = my; c->m[2] = mz;
  c->n = n;
  c->flags = flags;
  c->nranks = (int)nranks;
  c->sjy = (long)n * n * n * mx;
  c->sjz = jz_stride(n, mx, my);
  c->R = c->sjz * mz;
  c->total = c->R * nranks;
  c->nbr = neighbour_table(c->L, (flags & FACES_PERIODIC) != 0);
  c->msg_off.assign(nranks * 27, -1);
  if (flags & FACES_MESSAGES) c->msg_total = message_offsets(c->desc(nullptr), c->nbr, c->msg_off);
  if (flags & (FACES_V6 | FACES_V6F)) c->msg_total = v6_message_doubles(c->desc(nullptr));
  c->recv_off = receive_offsets(c->nbr, c->msg_off);
  cudaError_t e;
  if ((e = cudaMalloc(&c->d_nbr, sizeof(int) * nranks * 27)) != cudaSuccess ||
      (e = cudaMalloc(&c->d_off, sizeof(long) * nranks * 27)) != cudaSuccess ||
      (e = cudaMalloc(&c->d_roff, sizeof(long) * nranks * 27)) != cudaSuccess ||
      (e = cudaMalloc(&c->d_scratch, sizeof(unsigned long long) * (nranks + 4))) != cudaSuccess ||
      (e = cudaMalloc(&c->d_sync, sizeof(unsigned long long) * 2)) != cudaSuccess ||
      (e = cudaMemset(c->d_sync, 0, sizeof(unsigned long long) * 2)) != cudaSuccess ||
      (c->msg_total > 0 && (e = cudaMalloc(&c->d_msg, sizeof(double) * c->msg_total)) != cudaSuccess)) {
    faces_destroy(c);
    return cuda_fail(e, "faces_create: device allocation");
  }
  if ((e = cudaMemcpy(c->d_nbr, c->nbr.data(), sizeof(int) * nranks * 27, cudaMemcpyHostToDevice)) != cudaSuccess ||
      (e = cudaMemcpy(c->d_off, c->msg_off.data(), sizeof(long) * nranks * 27, cudaMemcpyHostToDevice)) != cudaSuccess ||
      (e = cudaMemcpy(c->d_roff, c->recv_off.data(), sizeof(long) * nranks * 27, cudaMemcpyHostToDevice)) !=
          cudaSuccess ||
      (c->d_msg && (e = cudaMemset(c->d_msg, 0, sizeof(double) * c->msg_total)) != cudaSuccess)) {
    faces_destroy(c);
    return cuda_fail(e, "faces_create: upload");
  }
  int dev = 0;
  if ((e = cudaGetDevice(&dev)) != cudaSuccess ||
      (e = cudaDeviceGetAttribute(&c->sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess) {
    faces_destroy(c);
    return cuda_fail(e, "faces_create: device query");
  }
  c->variant = default_variant(*c);
  replan(*c);
  *out = c;
  return FACES_OK;
}

int faces_destroy(faces_ctx *c)
{
  if (!c) return FACES_OK;
  cudaFree(c->d_nbr);
  cudaFree(c->d_off);
  cudaFree(c->d_roff);
  cudaFree(c->d_msg);
  cudaFree(c->d_scratch);
  cudaFree(c->d_sync);
  cudaFree(c->d_field);
  cudaFree(c->d_field2);
  cudaFree(c->d_field3);
  for (cudaStream_t st : {c->s_up, c->s_down, c->s_comp})
    if (st) cudaStreamDestroy(st);
  for (cudaEvent_t e : {c->ev_up[0], c->ev_up[1], c->ev_up[2], c->ev_done[0], c->ev_done[1], c->ev_done[2],
                        c->ev_free[0], c->ev_free[1], c->ev_free[2],
                        c->ev_fork, c->ev_join})
    if (e) cudaEventDestroy(e);
  delete c;
  return FACES_OK;
}

int faces_layout(const faces_ctx *c, long strides[6], long *rank_doubles, long *total_doubles)
{
  if (int rc = check_ctx(c)) return rc;
  if (strides) {
    const long n = c->n;
    strides[0] = 1;
    strides[1] = n;
    strides[2] = n * n;
    strides[3] = n * n * n;
    strides[4] = c->sjy;
    strides[5] = c->sjz;
  }
  if (rank_doubles) *rank_doubles = c->R;
  if (total_doubles) *total_doubles = c->total;
  return FACES_OK;
}

int faces_field_alloc(const faces_ctx *c, double **u)
{
  if (int rc = check_ctx(c)) return rc;
  if (!u) return fail(FACES_EINVAL, "null output pointer");
  *u = nullptr;
  CUDA_TRY(cudaMalloc(u, sizeof(double) * c->total), "faces_field_alloc");
  CUDA_TRY(cudaMemset(*u, 0, sizeof(double) * c->total), "faces_field_alloc: memset");
  return FACES_OK;
}

int faces_field_free(double *u)
{
  CUDA_TRY(cudaFree(u), "faces_field_free");
  return FACES_OK;
}

int faces_set_tuning(faces_ctx *c, int chunk, int width, int order)
{
  if (int rc = check_ctx(c)) return rc;
  if (order % 16 > 3)
    return fail(FACES_EINVAL, "order = %d: -1 (default), 0, 1, 2 + 16*chunks_per_unit, or 3 (warp tiles)", order);
  c->chunk = chunk > 0 ? chunk : 0;
  c->tpb = width > 0 ? width : 0;
  c->order = order;
  c->variant = default_variant(*c);
  replan(*c);
  return FACES_OK;
}

int faces_get_tuning(const faces_ctx *c, int *chunk, int *unit_chunks, int *blocks, int *kernel, int *order)
{
  if (int rc = check_ctx(c)) return rc;
  const bool seams = seam_step(*c);
  if (kernel) *kernel = seams ? 3 : c->variant;
  if (order) *order = seams ? c->splan.lean : c->tplan.order;
  if (chunk) *chunk = seams ? c->splan.chunk : c->tplan.chunk;
  if (unit_chunks) *unit_chunks = seams ? 1 : c->tplan.unit_chunks;
  if (blocks) *blocks = (int)(seams ? c->splan.grid : c->tgrid);
  return FACES_OK;
}

int faces_test_pack_wait(faces_ctx *c, int extra, long polls)
{
  if (int rc = check_ctx(c)) return rc;
  if (extra < 0 || extra > 1 || polls < 1) return fail(FACES_EINVAL, "extra %d (0 or 1), polls %ld (>= 1)", extra, polls);
  c->pack_wait_extra = extra;
  c->pack_wait_polls = polls;
  return FACES_OK;
}

int faces_status(faces_ctx *c, int *bits)
{
  if (int rc = check_ctx(c)) return rc;
  if (!bits) return fail(FACES_EINVAL, "null output pointer");
  int v[2] = {0, 0};
  CUDA_TRY(cudaMemcpy(v, c->d_sync + 1, sizeof(v), cudaMemcpyDeviceToHost), "status: read");
  CUDA_TRY(cudaMemset(c->d_sync + 1, 0, sizeof(unsigned long long)), "status: clear");
  *bits = v[0];
  return FACES_OK;
}

int faces_launches_per_share(const faces_ctx *c, int compute)
{
  if (int rc = check_ctx(c)) return rc;
  if (c->flags & FACES_V6) return c->nranks == 1 && !(c->flags & FACES_PERIODIC) ? 3 : 6;
  if (c->flags & FACES_V6F) return 4;
  if (compute && seam_step(*c) && c->splan.lean && c->splan.plane_items > 0) return 2;
  if (pack_in_tiles(*c, compute)) return 1;
  return (c->flags & FACES_MESSAGES) && !no_messages(*c) ? 2 : 1;
}

static int share_once(faces_ctx *c, double *u, int compute, cudaStream_t s)
{
  const FieldDesc f = c->desc(u);
  if (c->flags & FACES_V6) {
    CUDA_TRY(launch_v6(f, c->d_msg, compute, s), "v-6 kernel launch");
    return FACES_OK;
  }
  if (c->flags & FACES_V6F) {
    CUDA_TRY(launch_v6_fused(f, c->d_msg, compute, s), "fused v-6 kernel launch");
    return FACES_OK;
  }
  const bool fused = compute && !(c->flags & FACES_GATHER);
  const bool pack_fused = pack_in_tiles(*c, compute);
  if ((c->flags & FACES_MESSAGES) && !pack_fused && !no_messages(*c)) CUDA_TRY(launch_pack(f, s), "pack kernel launch");
  if (fused && seam_step(*c)) {
    CUDA_TRY(launch_seams(f, c->splan, s), "seam kernel launch");
    return FACES_OK;
  }
  if (fused && !(c->flags & FACES_ROWS) && c->variant != 2 && tile_kernel_supported(c->n)) {
    const bool general = (c->flags & FACES_GENERAL) || c->variant == 1;
    if (c->tplan.order == 3 && !general) {
      CUDA_TRY(launch_wtiles(f, c->tplan, c->tgrid, s), "warp tile kernel launch");
    } else if (pack_fused) {
      const PackGrid g = pack_grid(f);
      const PackFuse pf{g.gx,    g.gy, g.wide ? 1 : 0, c->d_sync, reinterpret_cast<int *>(c->d_sync + 1),
                        c->pack_wait_extra, c->pack_wait_polls};
      CUDA_TRY(launch_tiles(f, c->tplan, c->tgrid, s, general, &pf), "message-mode tile kernel launch");
    } else {
      CUDA_TRY(launch_tiles(f, c->tplan, c->tgrid, s, general), "tile kernel launch");
    }
  } else if (fused && row_kernel_supported(c->n))
    CUDA_TRY(launch_rows(f, c->plan, s), "row kernel launch");
  else
    CUDA_TRY(launch_gather(f, compute, s), "gather kernel launch");
  return FACES_OK;
}

int faces_share(faces_ctx *c, double *u, int compute, void *stream)
{
  if (int rc = check_ctx(c)) return rc;
  if (int rc = check_field(u)) return rc;
  return share_once(c, u, compute, static_cast<cudaStream_t>(stream));
}

int faces_share_n(faces_ctx *c, double *u, int compute, int nshares, void *stream)
{
  if (int rc = check_ctx(c)) return rc;
  if (int rc = check_field(u)) return rc;
  if (nshares < 0) return fail(FACES_EINVAL, "nshares = %d must not be negative", nshares);
  for (int i = 0; i < nshares; i++)
    if (int rc = share_once(c, u, compute, static_cast<cudaStream_t>(stream))) return rc;
  return FACES_OK;
}

int faces_autotune(faces_ctx *c, double *u, int compute, int trials, void *stream)
{
  if (int rc = check_ctx(c)) return rc;
  if (!u) return fail(FACES_EINVAL, "null field");
  if (trials < 1) trials = 3;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (!(compute && !(c->flags & (FACES_GATHER | FACES_ROWS | FACES_V6 | FACES_V6F | FACES_SEAMS)) &&
        tile_kernel_supported(c->n)))
    return 0;
  // candidates: elements per tile (default, half, double), units of one
  // chunk or half a column (order 2 + 16*u), resident blocks per SM
  const int k0 = c->tplan.chunk;
  const int ks[3] = {k0, k0 / 2, k0 * 2};
  const int orders[3] = {-1, 2 + 16, 3};
  const int widths[2] = {0, 2};
  cudaEvent_t e0, e1;
  CUDA_TRY(cudaEventCreate(&e0), "autotune: event");
  CUDA_TRY(cudaEventCreate(&e1), "autotune: event");
  float best = 1e30f;
  int bk = c->chunk, bo = c->order, bw = c->tpb, bv = c->variant, applied = 0, rc = FACES_OK;
  // shares per trial: at least `trials`, and enough for about 1 ms (the
  // current settings' share time, measured once), so that short shares are
  // not timed by their launch overhead and noise
  int reps = trials;
  {
    replan(*c);
    if ((rc = share_once(c, u, compute, s)) == FACES_OK) {
      cudaEventRecord(e0, s);
      for (int t = 0; t < trials && rc == FACES_OK; t++) rc = share_once(c, u, compute, s);
      cudaEventRecord(e1, s);
      applied += 1 + trials;
    }
    float ms = 0;
    if (rc == FACES_OK && cudaEventSynchronize(e1) == cudaSuccess && cudaEventElapsedTime(&ms, e0, e1) == cudaSuccess &&
        ms > 0) {
      const float per = ms / trials;
      const int want = (int)(1.0f / per) + 1;
      reps = want < trials ? trials : (want > 200 ? 200 : want);
    }
  }
  // time the current settings (kernel variant v) once; keep the fastest
  auto trial = [&](int v) {
    c->variant = v;
    replan(*c);
    if ((rc = share_once(c, u, compute, s))) return;  // warm-up
    cudaEventRecord(e0, s);
    for (int t = 0; t < reps && rc == FACES_OK; t++) rc = share_once(c, u, compute, s);
    cudaEventRecord(e1, s);
    applied += 1 + reps;
    if (rc) return;
    cudaError_t e = cudaEventSynchronize(e1);
    if (e != cudaSuccess) {
      rc = fail(FACES_ECUDA, "autotune: %s", cudaGetErrorString(e));
      return;
    }
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    if (ms < best) { best = ms; bk = c->chunk; bo = c->order; bw = c->tpb; bv = v; }
  };
  const bool periodic_step = (c->flags & FACES_PERIODIC) && !(c->flags & (FACES_MESSAGES | FACES_GENERAL));
  for (int ki = 0; ki < 3 && rc == FACES_OK; ki++) {
    if (ks[ki] < 1 || (ki > 0 && ks[ki] == k0)) continue;
    for (int o : orders)
      for (int w : widths) {
        if (rc != FACES_OK) break;
        if (o == 3 && (ki > 0 || !periodic_step)) continue;  // warp tiles: periodic step, one tile length
        c->chunk = ks[ki];
        c->order = o;
        c->tpb = w;
        replan(*c);
        if (ki == 2 && c->tplan.chunk == k0) continue;  // doubling not possible
        trial(0);
      }
  }
  // the other kernels at their default settings: the general tile step
  // (where the mixed step runs) and the row kernel
  c->chunk = 0;
  c->order = -1;
  c->tpb = 0;
  if (rc == FACES_OK && !periodic_step && !(c->flags & FACES_GENERAL)) trial(1);
  if (rc == FACES_OK && row_kernel_supported(c->n)) trial(2);
  // the seam kernel (direct mode): the chunked form (order 0) at its
  // default chunk (shortened for small fields) and at twice the unshortened
  // one, and the lean form (order 1)
  if ((!(c->flags & FACES_MESSAGES) || no_messages(*c)) && seam_kernel_supported(c->n)) {
    const int e0 = seam_default_chunk(c->n);
    c->order = 0;
    for (int e : {0, 2 * e0}) {
      if (rc != FACES_OK) break;
      c->chunk = e;
      trial(3);
    }
    c->chunk = 0;
    c->order = 1;
    if (rc == FACES_OK) trial(3);
    c->order = -1;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  c->chunk = bk;
  c->order = bo;
  c->tpb = bw;
  c->variant = bv;
  replan(*c);
  return rc ? rc : applied;
}

int faces_init_ref(faces_ctx *c, double *u, void *stream)
{
  if (int rc = check_ctx(c)) return rc;
  if (int rc = check_field(u)) return rc;
  CUDA_TRY(launch_init_ref(c->desc(u), static_cast<cudaStream_t>(stream)), "init kernel launch");
  return FACES_OK;
}

int faces_init_int(faces_ctx *c, double *u, unsigned long long seed, void *stream)
{
  if (int rc = check_ctx(c)) return rc;
  if (int rc = check_field(u)) return rc;
  CUDA_TRY(launch_init_int(c->desc(u), seed, static_cast<cudaStream_t>(stream)), "init kernel launch");
  return FACES_OK;
}

int faces_check(faces_ctx *c, const double *u, int init, unsigned long long seed, int nshares, int compute,
                double *rank_maxrel, double *maxrel, int *npass, int where[7], double vals[2], void *stream)
{
  if (int rc = check_ctx(c)) return rc;
  if (int rc = check_field(u)) return rc;
  if (init != 0 && init != 1) return fail(FACES_EINVAL, "init = %d: 0 (reference formula) or 1 (integer seed)", init);
  if (nshares < 0) return fail(FACES_EINVAL, "nshares = %d must not be negative", nshares);
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const int R = c->nranks;
  unsigned long long *rank_max = c->d_scratch, *gmax = c->d_scratch + R, *first = c->d_scratch + R + 1;
  double *dvals = reinterpret_cast<double *>(c->d_scratch + R + 2);
  const FieldDesc f = c->desc(const_cast<double *>(u));
  CUDA_TRY(cudaMemsetAsync(c->d_scratch, 0, sizeof(unsigned long long) * (R + 1), s), "check: clear");
  CUDA_TRY(cudaMemsetAsync(first, 0xff, sizeof(unsigned long long), s), "check: clear");
  CUDA_TRY(launch_check(f, init, seed, nshares, compute, rank_max, gmax, 0, first, -1, dvals, s), "check kernel");
  std::vector<unsigned long long> h(R + 1);
  CUDA_TRY(cudaMemcpyAsync(h.data(), c->d_scratch, sizeof(unsigned long long) * (R + 1), cudaMemcpyDeviceToHost, s),
           "check: read back");
  CUDA_TRY(cudaStreamSynchronize(s), "check: synchronize");
  int pass = 0;
  for (int r = 0; r < R; r++) {
    double d;
    std::memcpy(&d, &h[r], sizeof(d));
    if (rank_maxrel) rank_maxrel[r] = d;
    if (d < 1e-15) pass++;
  }
  double g;
  std::memcpy(&g, &h[R], sizeof(g));
  if (maxrel) *maxrel = g;
  if (npass) *npass = pass;
  if (where || vals) {
    long p = 0;
    if (h[R] != 0) {
      CUDA_TRY(launch_check(f, init, seed, nshares, compute, rank_max, gmax, h[R], first, -1, dvals, s), "check: locate");
      unsigned long long hp;
      CUDA_TRY(cudaMemcpyAsync(&hp, first, sizeof(hp), cudaMemcpyDeviceToHost, s), "check: read back");
      CUDA_TRY(cudaStreamSynchronize(s), "check: synchronize");
      p = (long)hp;
    }
    const long n = c->n;
    const long per_rank = n * n * n * c->m[0] * c->m[1] * c->m[2];
    const long points = per_rank * c->nranks;
    if (where && p >= points) {
      // a padding double: its rank and jz slab, the point coordinates -1
      const long pad = c->sjz - c->sjy * c->m[1], q = p - points;
      where[0] = (int)(q / (pad * c->m[2]));
      for (int a = 1; a < 6; a++) where[a] = -1;
      where[6] = (int)((q % (pad * c->m[2])) / pad);
    } else if (where) {
      long t = p % per_rank;
      where[0] = (int)(p / per_rank);
      where[1] = (int)(t % n); t /= n;
      where[2] = (int)(t % n); t /= n;
      where[3] = (int)(t % n); t /= n;
      where[4] = (int)(t % c->m[0]); t /= c->m[0];
      where[5] = (int)(t % c->m[1]); t /= c->m[1];
      where[6] = (int)t;
    }
    if (vals) {
      CUDA_TRY(launch_check(f, init, seed, nshares, compute, rank_max, gmax, 0, first, p, dvals, s), "check: values");
      CUDA_TRY(cudaMemcpyAsync(vals, dvals, 2 * sizeof(double), cudaMemcpyDeviceToHost, s), "check: read back");
      CUDA_TRY(cudaStreamSynchronize(s), "check: synchronize");
    }
  }
  return FACES_OK;
}

int faces_run_host(faces_ctx *c, const double *u_in, double *u_out, int compute, int nshares, void *stream)
{
  if (int rc = check_ctx(c)) return rc;
  if (!u_in || !u_out) return fail(FACES_EINVAL, "null host buffer");
  if (nshares < 0) return fail(FACES_EINVAL, "nshares = %d must not be negative", nshares);
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (!c->d_field) CUDA_TRY(cudaMalloc(&c->d_field, sizeof(double) * c->total), "faces_run_host: device field");
  const size_t bytes = sizeof(double) * c->total;
  CUDA_TRY(cudaMemcpyAsync(c->d_field, u_in, bytes, cudaMemcpyHostToDevice, s), "faces_run_host: upload");
  if (int rc = faces_share_n(c, c->d_field, compute, nshares, stream)) return rc;
  CUDA_TRY(cudaMemcpyAsync(u_out, c->d_field, bytes, cudaMemcpyDeviceToHost, s), "faces_run_host: download");
  CUDA_TRY(cudaStreamSynchronize(s), "faces_run_host: synchronize");
  return FACES_OK;
}

int faces_run_host_many(faces_ctx *c, int njobs, const double *const *u_in, double *const *u_out, int compute,
                        int nshares, void *stream)
{
  if (int rc = check_ctx(c)) return rc;
  if (njobs < 0) return fail(FACES_EINVAL, "njobs = %d must not be negative", njobs);
  if (nshares < 0) return fail(FACES_EINVAL, "nshares = %d must not be negative", nshares);
  if (njobs == 0) return FACES_OK;
  if (!u_in || !u_out) return fail(FACES_EINVAL, "null job array");
  for (int j = 0; j < njobs; j++) {
    if (!u_in[j] || !u_out[j]) return fail(FACES_EINVAL, "job %d: null host buffer", j);
    // an upload may run while an earlier job's download is in flight
    for (int i = 0; i < j; i++)
      if (u_in[j] == u_out[i]) return fail(FACES_EINVAL, "job %d reads the output of job %d", j, i);
  }
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const size_t bytes = sizeof(double) * c->total;
  if (!c->d_field) CUDA_TRY(cudaMalloc(&c->d_field, bytes), "faces_run_host_many: device field");
  if (njobs > 1 && !c->d_field2) CUDA_TRY(cudaMalloc(&c->d_field2, bytes), "faces_run_host_many: second field");
  if (njobs > 2 && !c->d_field3) CUDA_TRY(cudaMalloc(&c->d_field3, bytes), "faces_run_host_many: third field");
  if (!c->pipe_ready) {
    CUDA_TRY(cudaStreamCreateWithFlags(&c->s_up, cudaStreamNonBlocking), "faces_run_host_many: stream");
    CUDA_TRY(cudaStreamCreateWithFlags(&c->s_down, cudaStreamNonBlocking), "faces_run_host_many: stream");
    CUDA_TRY(cudaStreamCreateWithFlags(&c->s_comp, cudaStreamNonBlocking), "faces_run_host_many: stream");
    cudaEvent_t *evs[11] = {&c->ev_up[0],   &c->ev_up[1],   &c->ev_up[2],   &c->ev_done[0],
                            &c->ev_done[1], &c->ev_done[2], &c->ev_free[0], &c->ev_free[1],
                            &c->ev_free[2], &c->ev_fork,    &c->ev_join};
    for (cudaEvent_t *e : evs) CUDA_TRY(cudaEventCreateWithFlags(e, cudaEventDisableTiming), "faces_run_host_many: event");
    c->pipe_ready = true;
  }
  double *dev[3] = {c->d_field, c->d_field2, c->d_field3};
  // The shares run on the context's own non-blocking stream, not the
  // caller's: on the legacy default stream (0) the copies of neighbouring
  // jobs overlapped the shares only in part (C2 field, 8 jobs: 21.0 ms per
  // job against 18.2 on a non-blocking stream, 22.1 with no overlap).  All
  // three streams start after the caller's earlier work on `stream`.
  cudaStream_t sc = c->s_comp;
  CUDA_TRY(cudaEventRecord(c->ev_fork, s), "faces_run_host_many: fork");
  for (cudaStream_t st : {c->s_up, c->s_down, sc})
    CUDA_TRY(cudaStreamWaitEvent(st, c->ev_fork, 0), "faces_run_host_many: fork");
  // Job j+1's upload is enqueued before job j's download: the two copy
  // streams may share one hardware queue, and there an upload enqueued after
  // a download (which waits for its job's shares) would wait for those shares
  // too, and the next job's shares for it -- no overlap at all (seen: 22.9 ms
  // per job against 18.2 with the copies hidden).
  // Three device fields: job j reuses job j-3's once that job's download is
  // done, so an upload has two jobs' shares to finish behind the downloads
  // (copies slow down while the shares load HBM; with two fields calls took
  // 18.2 to 22 ms per job).
  auto upload = [&](int j) -> int {
    const int b = j % 3;
    if (j >= 3) CUDA_TRY(cudaStreamWaitEvent(c->s_up, c->ev_free[b], 0), "faces_run_host_many: wait");
    CUDA_TRY(cudaMemcpyAsync(dev[b], u_in[j], bytes, cudaMemcpyHostToDevice, c->s_up), "faces_run_host_many: upload");
    CUDA_TRY(cudaEventRecord(c->ev_up[b], c->s_up), "faces_run_host_many: event");
    return FACES_OK;
  };
  if (int rc = upload(0)) return rc;
  for (int j = 0; j < njobs; j++) {
    const int b = j % 3;
    if (j + 1 < njobs)
      if (int rc = upload(j + 1)) return rc;
    CUDA_TRY(cudaStreamWaitEvent(sc, c->ev_up[b], 0), "faces_run_host_many: wait");
    if (int rc = faces_share_n(c, dev[b], compute, nshares, sc)) {
      // no copy or share of this call stays in flight behind an error
      for (cudaStream_t st : {c->s_up, c->s_down, sc}) cudaStreamSynchronize(st);
      return rc;
    }
    CUDA_TRY(cudaEventRecord(c->ev_done[b], sc), "faces_run_host_many: event");
    CUDA_TRY(cudaStreamWaitEvent(c->s_down, c->ev_done[b], 0), "faces_run_host_many: wait");
    CUDA_TRY(cudaMemcpyAsync(u_out[j], dev[b], bytes, cudaMemcpyDeviceToHost, c->s_down),
             "faces_run_host_many: download");
    CUDA_TRY(cudaEventRecord(c->ev_free[b], c->s_down), "faces_run_host_many: event");
  }
  // the caller's stream joins the downloads (and with them the uploads)
  CUDA_TRY(cudaEventRecord(c->ev_join, c->s_down), "faces_run_host_many: join");
  CUDA_TRY(cudaStreamWaitEvent(s, c->ev_join, 0), "faces_run_host_many: join");
  CUDA_TRY(cudaStreamSynchronize(s), "faces_run_host_many: synchronize");
  return FACES_OK;
}

}  // extern "C"
