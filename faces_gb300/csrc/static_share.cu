// static_share.cu -- faces_share_static: one message-mode share that
// allocates no device memory.
//
// Some callers cannot call cudaMalloc: applications that hand all of the
// GPU's memory to their own pool at start-up and forbid later allocations,
// and latency-critical loops that cannot afford the device-wide
// synchronisation cudaMalloc/cudaFree imply.  For them this entry point keeps
// its working memory -- the neighbour table, the message offsets and the 26
// message buffers of every rank -- in one file-scope device array of fixed
// size, kStaticScratchDoubles doubles (32 MiB), that every GPU which loads
// the library holds until the process exits.
//
// In host code the array's name is only a host-side stand-in, not a device
// address; the device address is taken once per device with
// cudaGetSymbolAddress, on that device's first call (so make the first call
// on a device before any stream capture).  The address is kept for the life
// of the process: a device reset (cudaDeviceReset, or the primary context
// released and created again) voids it, so a process that resets a device
// must not call this entry point on that device afterwards.  Each device has
// its own copy of the array.  Every call on a device uses that copy and
// leaves its contents behind: each call rewrites the tables and the messages
// before reading them.  Two calls that overlap on the same device (for
// example on two streams that are not ordered with each other) race on it.
#include <cuda_runtime.h>

#include <cstdarg>
#include <cstdint>
#include <cstdio>
#include <mutex>
#include <string>

#include "../../include/faces_gb300.h"
#include "geom.cuh"
#include "kernels.cuh"
#include "rows_setup.cuh"

using namespace faces;

namespace {

constexpr long kStaticScratchDoubles = FACES_STATIC_SCRATCH_DOUBLES;  // 32 MiB
constexpr int kMaxDevices = 64;

__device__ __align__(256) double g_static_scratch[kStaticScratchDoubles];

std::mutex g_setup_mu;
double *g_scratch_ptr[kMaxDevices] = {};

// Layout of the scratch for one call: nbr (int, nranks*27, rounded to whole
// doubles), msg_off and recv_off (long, nranks*27 each), then the messages.
// A rank's buffer toward direction dir sits at a fixed offset: rank *
// per_rank + dir_off[dir] whether or not that neighbour exists, so the
// offsets need no prefix sum.
struct StaticLayout {
  long nbr_d, off_d, msg_d, total_d;
  long per_rank;
  long dir_off[27];
};

StaticLayout static_layout(const FieldDesc &f)
{
  StaticLayout s;
  long o = 0;
  for (int dir = 0; dir < 27; dir++) {
    s.dir_off[dir] = o;
    if (dir == 13) continue;
    const int d[3] = {dir % 3 - 1, (dir / 3) % 3 - 1, dir / 9 - 1};
    o += (region_size(f, d) + 31) / 32 * 32;
  }
  s.per_rank = o;
  const long nr27 = 27L * f.nranks;
  s.nbr_d = (nr27 + 1) / 2;
  s.off_d = nr27;
  s.msg_d = s.per_rank * f.nranks;
  s.total_d = ((s.nbr_d + 31) / 32 * 32) + 2 * ((s.off_d + 31) / 32 * 32) + s.msg_d;
  return s;
}

struct DirOffsets {
  long v[27];
};

// neighbour table, send and receive offsets of every rank, written into the
// scratch
__global__ void static_tables_kernel(int *nbr, long *off, long *roff, int L0, int L1, int L2, int periodic,
                                     long per_rank, DirOffsets dir_off, int nranks)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nranks * 27) return;
  const int r = i / 27, dir = i % 27;
  const int L[3] = {L0, L1, L2};
  const int k[3] = {r % L0, (r / L0) % L1, r / (L0 * L1)};
  const int d[3] = {dir % 3 - 1, (dir / 3) % 3 - 1, dir / 9 - 1};
  int q[3];
  bool ok = true;
  for (int a = 0; a < 3; a++) {
    q[a] = k[a] + d[a];
    if (q[a] < 0 || q[a] >= L[a]) {
      if (!periodic) ok = false;
      q[a] = (q[a] + L[a]) % L[a];
    }
  }
  const int peer = (q[2] * L1 + q[1]) * L0 + q[0];
  nbr[i] = ok ? peer : -1;
  if (dir == 13) nbr[i] = r;
  off[i] = (ok && dir != 13) ? r * per_rank + dir_off.v[dir] : -1;
  roff[i] = (ok && dir != 13) ? peer * per_rank + dir_off.v[26 - dir] : -1;
}

}  // namespace

// sets faces_last_error()'s text (faces_api.cu)
void faces_internal_set_error(const char *msg);

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

// the scratch's device address on the current device (taken on first use)
int scratch_on_device(double **ptr)
{
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return fail(FACES_ECUDA, "faces_share_static: cudaGetDevice: %s", cudaGetErrorString(e));
  if (dev < 0 || dev >= kMaxDevices) return fail(FACES_EUNSUPPORTED, "faces_share_static: device %d", dev);
  std::lock_guard<std::mutex> lock(g_setup_mu);
  if (!g_scratch_ptr[dev]) {
    void *p = nullptr;
    e = cudaGetSymbolAddress(&p, g_static_scratch);
    if (e != cudaSuccess || !p)
      return fail(FACES_ECUDA, "faces_share_static: cudaGetSymbolAddress: %s", cudaGetErrorString(e));
    g_scratch_ptr[dev] = static_cast<double *>(p);
  }
  *ptr = g_scratch_ptr[dev];
  return FACES_OK;
}

}  // namespace

extern "C" int faces_share_static(double *u, int lx, int ly, int lz, int mx, int my, int mz, int n, unsigned flags,
                                  int compute, void *stream)
{
  if (!u) return fail(FACES_EINVAL, "faces_share_static: null field pointer");
  if ((reinterpret_cast<uintptr_t>(u) & 15u) != 0)
    return fail(FACES_EALIGN, "faces_share_static: field pointer is not 16-byte aligned");
  if (lx < 1 || ly < 1 || lz < 1 || mx < 1 || my < 1 || mz < 1 || n < 2)
    return fail(FACES_EINVAL, "faces_share_static: rank grid, element grid and n must be positive (n >= 2)");
  if (flags & ~FACES_PERIODIC)
    return fail(FACES_EINVAL, "faces_share_static: flags 0x%x: only FACES_PERIODIC applies", flags);
  const long nranks = (long)lx * ly * lz;
  if (nranks > 65535 / 27) return fail(FACES_EINVAL, "faces_share_static: %ld ranks: at most %d", nranks, 65535 / 27);

  FieldDesc f;
  f.u = u;
  f.n = n;
  f.m[0] = mx; f.m[1] = my; f.m[2] = mz;
  f.L[0] = lx; f.L[1] = ly; f.L[2] = lz;
  f.periodic = (flags & FACES_PERIODIC) ? 1 : 0;
  f.mode = kMessages;
  f.nranks = (int)nranks;
  f.sjy = (long)n * n * n * mx;
  f.sjz = jz_stride(n, mx, my);
  f.R = f.sjz * mz;

  const StaticLayout lay = static_layout(f);
  if (lay.total_d > kStaticScratchDoubles)
    return fail(FACES_EINVAL,
                "faces_share_static: this field needs %ld doubles of message scratch, the static scratch holds "
                "%ld (%ld MiB); use faces_share with FACES_MESSAGES",
                lay.total_d, kStaticScratchDoubles, kStaticScratchDoubles * 8 >> 20);

  double *scratch = nullptr;
  if (int rc = scratch_on_device(&scratch)) return rc;
  int *nbr = reinterpret_cast<int *>(scratch);
  long *off = reinterpret_cast<long *>(scratch + (lay.nbr_d + 31) / 32 * 32);
  long *roff = off + (lay.off_d + 31) / 32 * 32;
  double *msg = scratch + (lay.nbr_d + 31) / 32 * 32 + 2 * ((lay.off_d + 31) / 32 * 32);
  f.nbr = nbr;
  f.msg_off = off;
  f.recv_off = roff;
  f.msg = msg;

  cudaStream_t s = static_cast<cudaStream_t>(stream);
  DirOffsets dof;
  for (int d = 0; d < 27; d++) dof.v[d] = lay.dir_off[d];
  const int items = (int)nranks * 27;
  static_tables_kernel<<<(items + 255) / 256, 256, 0, s>>>(nbr, off, roff, lx, ly, lz, f.periodic, lay.per_rank,
                                                          dof, (int)nranks);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return fail(FACES_ECUDA, "faces_share_static: table kernel: %s", cudaGetErrorString(e));
  if ((e = launch_pack(f, s)) != cudaSuccess)
    return fail(FACES_ECUDA, "faces_share_static: pack kernel: %s", cudaGetErrorString(e));
  if (compute && tile_kernel_supported(n)) {
    int dev = 0, sms = 0;
    if ((e = cudaGetDevice(&dev)) != cudaSuccess ||
        (e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess)
      return fail(FACES_ECUDA, "faces_share_static: device query: %s", cudaGetErrorString(e));
    // the default plan of faces_share for a message-mode field: the field's
    // tile form, its default tile length (halved while the form's shared
    // memory exceeds 110 KB), units of half a column, the resident blocks per
    // SM that shared memory and the form's launch bounds allow
    const TileForm form = tile_form(f, false);
    int k = tile_default_chunk(n, form);
    while (k > 1 && tile_form_smem_bytes(n, k, form) > 110 * 1024) k /= 2;
    RowPlan p = make_row_plan(f, k, 0);
    p.order = 2;
    p.unit_chunks = (p.nchunks + 1) / 2;
    e = launch_tiles(f, p, (long)sms * tile_blocks_per_sm(n, k, form), s);
  } else {
    e = launch_gather(f, compute, s);
  }
  if (e != cudaSuccess) return fail(FACES_ECUDA, "faces_share_static: step kernel: %s", cudaGetErrorString(e));
  return FACES_OK;
}
