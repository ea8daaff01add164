// ptile_steps.cuh -- the tile step for direct-mode periodic fields.
//
// In a periodic field every tile is regular: every staged row exists, every
// row has its x-lower end, and no tile takes an x-upper end.  A row's
// source then needs no per-row setup: slot (sy, sz) of a tile of column
// (rank, jy, jz) is row (iy, iz) = (sy, sz) of the element in one of four
// columns -- (jy, jz), (jy-1, jz), (jy, jz-1), (jy-1, jz-1), chosen by
// sy == n-1 and sz == n-1, wrapping to the neighbour rank -- and its x-lower
// end is point n-1 of element jx0-1, or of element mx-1 of the x-lower
// neighbour rank for the first chunk.  Only the pieces the passes use are
// moved: both ends of the interior rows, the seam rows in full.  The shared-memory
// layout is the general tile step's, so the dense passes (sum_tile) are
// shared.  What each tile reads and writes is exactly what the general step
// reads and writes for a regular tile.
#pragma once

#include <cuda_runtime.h>

#include "geom.cuh"
#include "rows_setup.cuh"
#include "tile_ops.cuh"
#include "tile_steps.cuh"

namespace faces {

// offsets (doubles from the field base) of a tile's four columns at its
// first element and of their x-lower end elements; column s: bit 0 the
// y-lower column, bit 1 the z-lower column
struct PMeta {
  long off[4];
  long lo[4];
  double *u;  // the field (so that a tile's sums need no global read)
  double *pad;
};

// a field whose tiles the periodic step takes
FACES_HD bool ptile_field(const FieldDesc &f) { return f.periodic && f.mode == kDirect; }

namespace ptile {

using namespace tiledev;

template <int N>
__host__ __device__ __forceinline__ long col_off(const FieldDesc &f, const TileCursor &u, int s, bool xlower, int jx)
{
  const bool ly = (s & 1) != 0, lz = (s & 2) != 0;
  const int dy = (ly && u.jy == 0) ? -1 : 0, dz = (lz && u.jz == 0) ? -1 : 0, dx = xlower ? -1 : 0;
  const int jy = ly ? (u.jy == 0 ? f.m[1] - 1 : u.jy - 1) : u.jy;
  const int jz = lz ? (u.jz == 0 ? f.m[2] - 1 : u.jz - 1) : u.jz;
  int q = u.r;
  if (f.nranks > 1 && (dx | dy | dz)) {
#ifdef __CUDA_ARCH__
    q = __ldg(f.nbr + u.r * 27 + dir_index(dx, dy, dz));
#else
    q = f.nbr[u.r * 27 + dir_index(dx, dy, dz)];
#endif
  }
  return (long)q * f.R + (long)jz * f.sjz + (long)jy * f.sjy + (long)jx * (N * N * N);
}

// the column of slot r
template <int N>
__host__ __device__ __forceinline__ int col_sel(int sy, int sz)
{
  return (sy == N - 1 ? 1 : 0) | (sz == N - 1 ? 2 : 0);
}

// The pieces a tile moves per element: the two end pieces of each interior
// row (1 <= sy, sz <= n-2), then every piece of each seam row.  Item j of an
// element -> row (sy, sz) and piece pc.
template <int N>
struct Needed {
  static constexpr int NP = pieces_per_row(N), NI = (N - 2) * (N - 2), NB = N * N - NI;
  static constexpr int count = NI * (NP > 1 ? 2 : 1) + NB * NP;
};

template <int N>
__host__ __device__ __forceinline__ void needed_piece(int j, int &sy, int &sz, int &pc)
{
  constexpr int NP = Needed<N>::NP, NI = Needed<N>::NI, E = NP > 1 ? 2 : 1;
  if constexpr (NI > 0) {
    if (j < NI * E) {
      const int ri = j / E;
      pc = (j - ri * E) ? NP - 1 : 0;
      sy = 1 + ri % (N - 2);
      sz = 1 + ri / (N - 2);
      return;
    }
  }
  j -= NI * E;
  const int b = j / NP;
  pc = j - b * NP;
  if (b < N) { sy = b; sz = 0; }
  else if (b < 2 * N) { sy = b - N; sz = N - 1; }
  else {
    const int t = b - 2 * N;
    sz = 1 + t / 2;
    sy = (t & 1) ? N - 1 : 0;
  }
}

// A team of T threads (a block of 256, or one warp) works on a tile; t is
// the thread's index in its team.  The functions also compile for the host,
// where tests/native/ptile_emu.cu replays them thread by thread.  Threads and needed slots: with more than
// T/2 slots per element thread t takes slots t, t+T, ... (SPT of them) for
// every element of the tile; with fewer, KT = T/slots threads share a slot
// and thread t takes its elements t/slots, +KT, ...  A thread decodes its
// slot once per tile and walks the elements by adding the element stride.
template <int N, int T>
struct PSlots {
  static constexpr int NE = Needed<N>::count;
  static constexpr int KT = NE <= T / 2 ? T / NE : 1;
  static constexpr int SPT = KT > 1 ? 1 : (NE + T - 1) / T;
};

template <int N, int T>
__host__ __device__ __forceinline__ bool pslot(int jj, int t, int &j, int &kq)
{
  constexpr int NE = PSlots<N, T>::NE, KT = PSlots<N, T>::KT;
  if constexpr (KT > 1) {
    j = t % NE;
    kq = t / NE;
    return kq < KT;
  } else {
    j = t + jj * T;
    kq = 0;
    return j < NE;
  }
}

// Stage tile u: the needed pieces of its elements, and the x-lower ends.
template <int N, int K, int T = 256>
__host__ __device__ __forceinline__ void pstage(const FieldDesc &fd, const RowPlan &p, const TileCursor &u, double *buf,
                                       PMeta *meta, int4 *tinfo, int t)
{
  // one copy of the description (the batched kernel reads it from global
  // memory; stores through double pointers must not force it to reload)
  const FieldDesc f = fd;
  constexpr int NN = N * N, PW = piece_doubles(N), RS = smem_row_stride(N);
  constexpr int KT = PSlots<N, T>::KT, SPT = PSlots<N, T>::SPT;
  constexpr long N3 = (long)N * N * N;
  const int jx0 = u.c * p.chunk;
  const int nk = p.chunk < f.m[0] - jx0 ? p.chunk : f.m[0] - jx0;
  const bool first = u.c == 0;
  const int jxl = first ? f.m[0] - 1 : jx0 - 1;
  if (t < 4) {
    meta->off[t] = col_off<N>(f, u, t, false, jx0);
    meta->lo[t] = col_off<N>(f, u, t, first, jxl);
  }
  if (t == 4) meta->u = f.u;
  if (t == 0) *tinfo = make_int4(jx0, nk, 0, 0);
  const long o0 = col_off<N>(f, u, 0, false, jx0), o1 = col_off<N>(f, u, 1, false, jx0);
  const long o2 = col_off<N>(f, u, 2, false, jx0), o3 = col_off<N>(f, u, 3, false, jx0);
#pragma unroll
  for (int jj = 0; jj < SPT; jj++) {
    int j, kq;
    if (!pslot<N, T>(jj, t, j, kq)) continue;
    int sy, sz, pc;
    needed_piece<N>(j, sy, sz, pc);
    const int s = col_sel<N>(sy, sz);
    const long o = s == 0 ? o0 : s == 1 ? o1 : s == 2 ? o2 : o3;
    const double *g = f.u + o + kq * N3 + sz * NN + sy * N + pc * PW;
    double *sp = buf + (kq * NN + sz * N + sy) * RS + pc * PW;
    for (int k = kq; k < nk; k += KT, g += KT * N3, sp += KT * NN * RS) cp_async(sp, g, PW);
  }
  for (int r = t; r < NN; r += T) {
    const int sy = r % N, sz = r / N;
    const long ol = col_off<N>(f, u, col_sel<N>(sy, sz), first, jxl);
    cp_async(buf + K * NN * RS + r, f.u + ol + sz * NN + sy * N + (N - 1), 1);
  }
  cp_commit();
}

// Sums of a staged tile, each final value stored as soon as it is known:
//   pxpass  -- x pairs (element k-1 at n-1, or the x-lower end, with element
//              k at 0) on every row; an interior row's pair is final there;
//   pyzpass -- after a barrier: y pairs of rows (0, o), (n-1, o) and z pairs
//              of rows (o, 0), (o, n-1) for o in 1..n-2, and the four corner
//              rows (y pairs, then z pairs), column by column.  These cells
//              are disjoint, so one phase does them all.
// The order is the general step's (x, then y, then z pairs) and every stored
// cell is one the general step stores, without the unchanged ones.
template <int N, int K, int T = 256>
__host__ __device__ __forceinline__ void pxpass(double *__restrict__ u, double *buf, const PMeta *meta, int nk, int t)
{
  constexpr int NN = N * N, RS = smem_row_stride(N);
  constexpr long N3 = (long)N * N * N;
  double *locol = buf + K * NN * RS;
  const int items = nk * NN;
  for (int i = t; i < items; i += T) {
    const int k = i / NN, r = i - k * NN;
    double *lo = k == 0 ? locol + r : buf + ((k - 1) * NN + r) * RS + (N - 1);
    double *hi = buf + (k * NN + r) * RS;
    const double s = *lo + *hi;
    *lo = s;
    *hi = s;
    const int sy = r % N, sz = r / N;
    if (sy >= 1 && sy <= N - 2 && sz >= 1 && sz <= N - 2) {
      // interior rows lie in column 0 (the tile's own elements)
      double *g = u + meta->off[0] + k * N3 + sz * NN + sy * N;
      g[0] = s;
      if (k == 0) u[meta->lo[0] + sz * NN + sy * N + (N - 1)] = s;
      else g[-N3 + (N - 1)] = s;
    }
  }
}

template <int N, int K, int T = 256>
__host__ __device__ __forceinline__ void pyzpass(double *__restrict__ u, const double *buf, const PMeta *meta, int nk, int t)
{
  constexpr int NN = N * N, RS = smem_row_stride(N);
  constexpr long N3 = (long)N * N * N;
  constexpr int G = 2 * (N - 2) + 1, COLS = K * N + 1;
  const double *locol = buf + K * NN * RS;
  const int last_c = (nk - 1) * N + (N - 1);  // the next chunk's seam: not stored
  for (int i = t; i < G * COLS; i += T) {
    const int g = i / COLS, c = i - g * COLS;
    const double *sb;
    int srs;
    long gcol;  // offset of the column within its row, and which offsets table
    bool lo = false;
    if (c < K * N) {
      const int k = c / N, x = c - k * N;
      if (k >= nk) continue;
      sb = buf + k * NN * RS + x;
      srs = RS;
      gcol = k * N3 + x;
    } else {
      sb = locol;
      srs = 1;
      gcol = N - 1;
      lo = true;
    }
    const bool store = lo || c != last_c;
    const long *offs = lo ? meta->lo : meta->off;
    auto gaddr = [&](int sy, int sz) { return u + offs[col_sel<N>(sy, sz)] + gcol + sz * NN + sy * N; };
    if (g < 2 * (N - 2)) {
      int ay, az, by, bz;
      if (g < N - 2) { ay = N - 1; by = 0; az = bz = 1 + g; }              // y pair
      else { ay = by = 1 + g - (N - 2); az = N - 1; bz = 0; }              // z pair
      const double s = sb[(az * N + ay) * srs] + sb[(bz * N + by) * srs];
      if (store) {
        *gaddr(ay, az) = s;
        *gaddr(by, bz) = s;
      }
    } else {
      const double c00 = sb[0], c10 = sb[(N - 1) * srs];
      const double c01 = sb[(N - 1) * N * srs], c11 = sb[(NN - 1) * srs];
      const double y0 = c10 + c00, y1 = c11 + c01;
      const double s = y1 + y0;
      if (store) {
        *gaddr(0, 0) = s;
        *gaddr(N - 1, 0) = s;
        *gaddr(0, N - 1) = s;
        *gaddr(N - 1, N - 1) = s;
      }
    }
  }
}

}  // namespace ptile
}  // namespace faces
