// seams.cu -- the seam step (seam_steps.cuh) for direct-mode fields: a
// thread per shared point, no shared memory.  Two forms:
//   chunked  one launch; persistent blocks walk x-chunks of a column, a
//            thread takes slots of the chunk (all three planes' points);
//   lean     one thread per face slot of the field, which also takes the
//            edge points (and the corner) at its coordinate: few registers,
//            many resident warps; a second launch for the open boundary
//            planes of a non-periodic field.
#include <cuda_runtime.h>

#include <atomic>

#include "kernels.cuh"
#include "seam_steps.cuh"

namespace faces {

namespace {

constexpr int kSeamThreads = 256;

// chunked: blocks walk the chunks (grid-stride), then every thread takes
// items of the open upper boundary planes (grid-stride).  The two sets of
// points are disjoint, so nothing orders them.
template <int N>
__global__ void __launch_bounds__(kSeamThreads, 4) seam_kernel(FieldDesc f, int E, int nch, long units, long plane_items)
{
  constexpr int S = seam_slots(N);
  for (long w = blockIdx.x; w < units; w += gridDim.x) {
    const SeamUnit un = seam_unit(f, E, nch, w);
    const SeamChunk c = seam_chunk<N>(f, un.r, un.jy, un.jz, un.jx0, un.nk);
    const int items = un.nk * S;
    for (int q = threadIdx.x; q < items; q += kSeamThreads) seam_item<N>(f.u, c, q);
  }
  for (long p = (long)blockIdx.x * kSeamThreads + threadIdx.x; p < plane_items; p += (long)gridDim.x * kSeamThreads)
    seam_plane_point(f, p);
}

// lean: one face slot per thread (with its edge points); blockIdx.x is the
// position along the column, so that consecutive blocks take consecutive
// elements of one column (an element's x-lower neighbour is still in cache),
// and blockIdx.y + gridDim.y * blockIdx.z the column (rank, jz, jy)
template <int N>
__global__ void __launch_bounds__(kSeamThreads, 6) seam_lean_kernel(FieldDesc f, int per_column)
{
  const int t = blockIdx.x * kSeamThreads + threadIdx.x;
  if (t < per_column) seam_lean_item<N>(f, (int)(blockIdx.y + gridDim.y * blockIdx.z), t);
}

// lean: the open boundary planes
__global__ void __launch_bounds__(kSeamThreads) seam_plane_kernel(FieldDesc f, long items)
{
  for (long g = (long)blockIdx.x * kSeamThreads + threadIdx.x; g < items; g += (long)gridDim.x * kSeamThreads)
    seam_plane_point(f, g);
}

template <int N>
int blocks_per_sm_n()
{
  // per device: the occupancy query runs once per device and n
  static std::atomic<int> cache[64];
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) dev = 0;
  int b = cache[dev].load();
  if (b > 0) return b;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, seam_kernel<N>, kSeamThreads, 0) != cudaSuccess || b < 1) b = 1;
  cache[dev].store(b);
  return b;
}

long blocks_for(long items, long cap)
{
  const long b = (items + kSeamThreads - 1) / kSeamThreads;
  return b < 1 ? 1 : (b > cap ? cap : b);
}

template <int N>
cudaError_t launch_n(const FieldDesc &f, const SeamPlan &p, cudaStream_t s)
{
  if (p.lean) {
    // columns as y (up to 65535) times z: cols = gy * gz exactly
    const long cols = (long)f.nranks * f.m[1] * f.m[2];
    const long per_column = (long)f.m[0] * seam_lean_slots(N);
    const long xs = (per_column + kSeamThreads - 1) / kSeamThreads;
    long gy = cols, gz = 1;
    if (cols > 65535) {
      gy = f.m[1];
      gz = cols / f.m[1];
    }
    if (gy > 65535 || gz > 65535 || per_column > 0x7fffffffL) return cudaErrorInvalidConfiguration;
    seam_lean_kernel<N><<<dim3((unsigned)xs, (unsigned)gy, (unsigned)gz), kSeamThreads, 0, s>>>(f, (int)per_column);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess || p.plane_items == 0) return e;
    seam_plane_kernel<<<(unsigned)blocks_for(p.plane_items, 1L << 16), kSeamThreads, 0, s>>>(f, p.plane_items);
    return cudaGetLastError();
  }
  if (p.units + p.plane_items == 0) return cudaSuccess;
  seam_kernel<N><<<(unsigned)p.grid, kSeamThreads, 0, s>>>(f, p.chunk, p.nch, p.units, p.plane_items);
  return cudaGetLastError();
}

}  // namespace

bool seam_kernel_supported(int n) { return n >= 2 && n <= 16; }

int seam_default_chunk(int n)
{
  // about eight slots per thread of a block per chunk
  const int e = 8 * kSeamThreads / seam_slots(n);
  return e < 1 ? 1 : e;
}

int seam_blocks_per_sm(int n)
{
  switch (n) {
    case 2: return blocks_per_sm_n<2>();
    case 3: return blocks_per_sm_n<3>();
    case 4: return blocks_per_sm_n<4>();
    case 5: return blocks_per_sm_n<5>();
    case 6: return blocks_per_sm_n<6>();
    case 7: return blocks_per_sm_n<7>();
    case 8: return blocks_per_sm_n<8>();
    case 9: return blocks_per_sm_n<9>();
    case 10: return blocks_per_sm_n<10>();
    case 11: return blocks_per_sm_n<11>();
    case 12: return blocks_per_sm_n<12>();
    case 13: return blocks_per_sm_n<13>();
    case 14: return blocks_per_sm_n<14>();
    case 15: return blocks_per_sm_n<15>();
    case 16: return blocks_per_sm_n<16>();
    default: return 1;
  }
}

SeamPlan make_seam_plan(const FieldDesc &f, int chunk, long grid, int lean)
{
  SeamPlan p;
  p.lean = lean;
  int e = chunk > 0 ? chunk : seam_default_chunk(f.n);
  if (e > f.m[0]) e = f.m[0];
  if (chunk <= 0) {
    // small fields: shorter chunks until there are two per block
    const long cols = (long)f.nranks * f.m[2] * f.m[1];
    while (e > 1 && cols * ((f.m[0] + e - 1) / e) < 2 * grid) e = (e + 1) / 2;
  }
  p.chunk = e;
  p.nch = (f.m[0] + e - 1) / e;
  p.units = (long)f.nranks * f.m[2] * f.m[1] * p.nch;
  // a non-periodic grid always has ranks with an open upper plane
  p.plane_items = f.periodic ? 0 : (long)f.nranks * seam_plane_items(f);
  p.grid = grid < 1 ? 1 : grid;
  return p;
}

cudaError_t launch_seams(const FieldDesc &f, const SeamPlan &p, cudaStream_t s)
{
  switch (f.n) {
    case 2: return launch_n<2>(f, p, s);
    case 3: return launch_n<3>(f, p, s);
    case 4: return launch_n<4>(f, p, s);
    case 5: return launch_n<5>(f, p, s);
    case 6: return launch_n<6>(f, p, s);
    case 7: return launch_n<7>(f, p, s);
    case 8: return launch_n<8>(f, p, s);
    case 9: return launch_n<9>(f, p, s);
    case 10: return launch_n<10>(f, p, s);
    case 11: return launch_n<11>(f, p, s);
    case 12: return launch_n<12>(f, p, s);
    case 13: return launch_n<13>(f, p, s);
    case 14: return launch_n<14>(f, p, s);
    case 15: return launch_n<15>(f, p, s);
    case 16: return launch_n<16>(f, p, s);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace faces
