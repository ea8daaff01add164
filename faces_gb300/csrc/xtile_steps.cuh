// xtile_steps.cuh -- the tile step for v-26 message mode (and one open rank).
//
// In message mode every rank sums each point of its subdomain boundary from
// its own copies and the copies its neighbours sent (the 26 messages of
// gpu/v-26-messages/Faces.cc:175-293, received by direction), and writes
// only its own copies (gpu/v-26-messages/Faces.cc:421-669).  The tiles are
// the general step's: x-chunks of the element columns (rank, jy, jz) with
// jy in [0, my] and jz in [0, mz] -- jy = my and jz = mz are the virtual top
// tiles whose row 0 is the upper neighbour's -- and the last chunk of a
// column takes the extra seam with the x-upper neighbour's element 0.
//
// In a periodic field every neighbour exists, so each tile is as regular as
// the periodic direct step's (ptile_steps.cuh): slot (sy, sz) is row
// (sy, sz) of one of four columns -- (jy, jz), (jy-1, jz), (jy, jz-1),
// (jy-1, jz-1) by sy == n-1 and sz == n-1 -- and a column outside
// [0, my) x [0, mz) is a received message: the face message from (0, dy, 0)
// or (0, 0, dz), rows of n doubles at element stride n^2, or the x-edge
// message from (0, dy, dz), rows at element stride n.  The x-lower ends of
// the first chunk and the x-upper ends of the last come from the messages
// of (-1, dy, dz) and (+1, dy, dz).  The only irregularity: in a virtual top
// tile the rows 1..n-2 along that axis do not exist (the neighbour keeps
// them), and no item touches them.
//
// Sums are the periodic step's passes in the same order (x pairs, then y,
// then z; lower copy first), so every rank computes the same bits for a
// shared point as its neighbours do, and the same bits as direct mode.
//
// Open fields (OPEN = true): the reference's own mode, where neighbour() is
// MPI_PROC_NULL outside the rank grid (gpu/v-26-messages/Faces.cc:92-103).
// A column or x end whose neighbour does not exist is absent: its rows are
// not staged, and a pair or corner sums only the copies that exist, in the
// same tree order (what gpu/Mugs.cc:86-416 computes at a global boundary).
// Both message-mode fields and one-rank direct-mode fields (which have no
// neighbour to read or write) take this form.
#pragma once

#include <cuda_runtime.h>

#include "geom.cuh"
#include "ptile_steps.cuh"
#include "rows_setup.cuh"
#include "tile_ops.cuh"
#include "tile_steps.cuh"

namespace faces {

// a field whose tiles this step takes: message mode, or one open rank
FACES_HD bool xtile_field(const FieldDesc &f)
{
  return f.mode == kMessages || (f.nranks == 1 && !f.periodic);
}

// The record of one tile, written one pipeline step before its copies are
// issued (so that the table loads behind its addresses are off the copies'
// path): for column s (bit 0 the y-lower column, bit 1 the z-lower one) the
// address of row (0, 0), point 0 of element jx0 and the strides of an
// element, a y row and a z row (0 along an axis the message does not span);
// the same for the x-lower and x-upper ends (point n-1 of element jx0-1, or
// the received end).  A null address is an absent column or end (open
// fields only).  wcol / wlo: bit s set where the column / lower end is the
// rank's own memory (written back; own columns lie in the field at its
// constant strides).  flags: hx (the last chunk: it takes the upper seam),
// vy, vz (virtual top tiles).
struct XMeta {
  double *col[4];
  double *lo[4];
  double *hi[4];
  int es[4], ys[4], zs[4];
  int lys[4], lzs[4], hys[4], hzs[4];
  int wcol, wlo, jx0, nk, flags, pad_[3];
};

namespace xtile {

using namespace tiledev;

struct XCol {
  double *base;
  int es, ys, zs;
  bool own;
};

struct XEnd {
  double *base;
  int ys, zs;
  bool own;
};

#ifdef __CUDA_ARCH__
#define FACES_XLDG(p) __ldg(p)
#else
#define FACES_XLDG(p) (*(p))
#endif

// the message rank r received from direction (dx, dy, dz); null where that
// neighbour does not exist, and in direct mode (one open rank: none does)
__host__ __device__ __forceinline__ double *recv(const FieldDesc &f, int r, int dx, int dy, int dz)
{
  if (f.mode != kMessages) return nullptr;
  const long o = FACES_XLDG(f.recv_off + r * 27 + dir_index(dx, dy, dz));
  return o < 0 ? nullptr : f.msg + o;
}

// the y or z offset of column s: -1 below the rank, +1 above (virtual top
// tile), and the element index inside the rank or the neighbour
__host__ __device__ __forceinline__ void col_axis(int j, int m, int &d, int &e)
{
  d = j < 0 ? -1 : (j >= m ? 1 : 0);
  e = j < 0 ? m - 1 : (j >= m ? 0 : j);
}

template <int N>
__host__ __device__ __forceinline__ XCol column(const FieldDesc &f, const TileCursor &u, int jx0, int s)
{
  constexpr long NN = N * N, N3 = NN * N;
  int dy, ey, dz, ez;
  col_axis(u.jy - (s & 1), f.m[1], dy, ey);
  col_axis(u.jz - ((s >> 1) & 1), f.m[2], dz, ez);
  XCol c;
  if (dy == 0 && dz == 0) {
    c.base = f.u + (long)u.r * f.R + (long)ez * f.sjz + (long)ey * f.sjy + jx0 * N3;
    c.es = (int)N3;
    c.ys = N;
    c.zs = (int)NN;
    c.own = true;
    return c;
  }
  double *m = recv(f, u.r, 0, dy, dz);
  c.own = false;
  if (!m) {
    c.base = nullptr;
    c.es = c.ys = c.zs = 0;
  } else if (dy != 0 && dz != 0) {  // x edge: ix + n*jx
    c.base = m + (long)jx0 * N;
    c.es = N;
    c.ys = c.zs = 0;
  } else if (dy != 0) {  // y face: ix + n*iz + n^2*jx + n^2*mx*jz
    c.base = m + NN * f.m[0] * ez + jx0 * NN;
    c.es = (int)NN;
    c.ys = 0;
    c.zs = N;
  } else {  // z face: ix + n*iy + n^2*jx + n^2*mx*jy
    c.base = m + NN * f.m[0] * ey + jx0 * NN;
    c.es = (int)NN;
    c.ys = N;
    c.zs = 0;
  }
  return c;
}

// the x end of column s on side dx (-1: lower, +1: upper) as a received
// message: the neighbour's plane x = its boundary, free axes y and/or z
template <int N>
__host__ __device__ __forceinline__ XEnd recv_end(const FieldDesc &f, const TileCursor &u, int s, int dx)
{
  constexpr long NN = N * N;
  int dy, ey, dz, ez;
  col_axis(u.jy - (s & 1), f.m[1], dy, ey);
  col_axis(u.jz - ((s >> 1) & 1), f.m[2], dz, ez);
  double *m = recv(f, u.r, dx, dy, dz);
  XEnd e;
  e.own = false;
  if (!m) {
    e.base = nullptr;
    e.ys = e.zs = 0;
  } else if (dy == 0 && dz == 0) {  // x face: iy + n*iz + n^2*jy + n^2*my*jz
    e.base = m + NN * ey + NN * f.m[1] * ez;
    e.ys = 1;
    e.zs = N;
  } else if (dy != 0 && dz != 0) {  // corner
    e.base = m;
    e.ys = e.zs = 0;
  } else if (dy != 0) {  // z edge: iz + n*jz
    e.base = m + (long)N * ez;
    e.ys = 0;
    e.zs = 1;
  } else {  // y edge: iy + n*jy
    e.base = m + (long)N * ey;
    e.ys = 1;
    e.zs = 0;
  }
  return e;
}

// the x-lower end of column s: point n-1 of element jx0-1 inside the
// column, or the received end for the first chunk
template <int N>
__host__ __device__ __forceinline__ XEnd lower_end(const FieldDesc &f, const TileCursor &u, const XCol &c, int s)
{
  if (u.c == 0) return recv_end<N>(f, u, s, -1);
  XEnd e;
  e.base = c.base ? c.base - c.es + (N - 1) : nullptr;
  e.ys = c.ys;
  e.zs = c.zs;
  e.own = c.own;
  return e;
}

// rows that exist: in a virtual top tile (jy = my or jz = mz) the rows
// 1..n-2 along that axis belong to the neighbour; in an open field, rows of
// an absent column do not exist either
template <int N, bool OPEN>
__host__ __device__ __forceinline__ bool row_exists(int sy, int sz, bool vy, bool vz, int pcol)
{
  return !(vy && sy >= 1 && sy <= N - 2) && !(vz && sz >= 1 && sz <= N - 2) &&
         (!OPEN || ((pcol >> ptile::col_sel<N>(sy, sz)) & 1));
}

// a + b over the copies that exist (pa, pb), the lower copy first
__host__ __device__ __forceinline__ double psum(double a, bool pa, double b, bool pb)
{
  return pa ? (pb ? a + b : a) : b;
}

// Describe tile u into its record, nine jobs: 0..3 the columns and their
// lower ends, 4..7 the upper ends, 8 the flags.  Job j < 8 runs on thread
// j*T/8 (one per warp of a block, so that their table loads wait in
// parallel), job 8 on thread 1; the other threads of the team do nothing.
template <int N, bool OPEN, int T = 256>
__host__ __device__ __forceinline__ void xdescribe(const FieldDesc &f, const RowPlan &p, const TileCursor &u,
                                                   XMeta *rec, int thread)
{
  static_assert(T % 8 == 0 && T / 8 >= 2, "eight describe jobs on distinct threads, and thread 1");
  const int t = thread == 1 ? 8 : (thread % (T / 8) == 0 ? thread / (T / 8) : -1);
  if (t < 0) return;
  const int jx0 = u.c * p.chunk;
  const bool hx = u.c == p.nchunks - 1;
  if (t < 4) {
    const XCol c = column<N>(f, u, jx0, t);
    rec->col[t] = c.base;
    rec->es[t] = c.es;
    rec->ys[t] = c.ys;
    rec->zs[t] = c.zs;
    const XEnd e = lower_end<N>(f, u, c, t);
    rec->lo[t] = e.base;
    rec->lys[t] = e.ys;
    rec->lzs[t] = e.zs;
  } else if (t < 8) {
    const int s = t - 4;
    const XEnd e = hx ? recv_end<N>(f, u, s, 1) : XEnd{nullptr, 0, 0, false};
    rec->hi[s] = e.base;
    rec->hys[s] = e.ys;
    rec->hzs[s] = e.zs;
  } else {
    // own columns: (jy', jz') inside the rank; their lower ends are own
    // past the first chunk
    int own = 0;
    for (int s = 0; s < 4; s++) {
      const int jy = u.jy - (s & 1), jz = u.jz - ((s >> 1) & 1);
      if (jy >= 0 && jy < f.m[1] && jz >= 0 && jz < f.m[2]) own |= 1 << s;
    }
    rec->wcol = own;
    rec->wlo = u.c > 0 ? own : 0;
    rec->jx0 = jx0;
    rec->nk = p.chunk < f.m[0] - jx0 ? p.chunk : f.m[0] - jx0;
    rec->flags = (hx ? 1 : 0) | (u.jy == f.m[1] ? 2 : 0) | (u.jz == f.m[2] ? 4 : 0);
  }
}

// A tile that reads no message and writes no point of the rank's boundary
// (what the pack reads): its four columns and their lower ends are the
// rank's own (not a first chunk), and it is not its column's last chunk.
__host__ __device__ __forceinline__ bool interior(const XMeta *rec)
{
  return rec->wcol == 15 && rec->wlo == 15 && !(rec->flags & 1);
}

// presence bits of a described tile's columns and lower ends (all, in a
// periodic field)
template <bool OPEN>
__host__ __device__ __forceinline__ int present_columns(const XMeta *rec)
{
  if (!OPEN) return 15;
  return (rec->col[0] ? 1 : 0) | (rec->col[1] ? 2 : 0) | (rec->col[2] ? 4 : 0) | (rec->col[3] ? 8 : 0);
}

template <bool OPEN>
__host__ __device__ __forceinline__ int present_lower_ends(const XMeta *rec)
{
  if (!OPEN) return 15;
  return (rec->lo[0] ? 1 : 0) | (rec->lo[1] ? 2 : 0) | (rec->lo[2] ? 4 : 0) | (rec->lo[3] ? 8 : 0);
}

// every column and x end of the tile exists (a periodic field: always; an
// open one: away from the global boundary); such tiles take the passes'
// periodic form
template <bool OPEN>
__host__ __device__ __forceinline__ bool complete(const XMeta *rec)
{
  if (!OPEN) return true;
  const bool hx = (rec->flags & 1) != 0;
  return present_columns<true>(rec) == 15 && present_lower_ends<true>(rec) == 15 &&
         (!hx || (rec->hi[0] && rec->hi[1] && rec->hi[2] && rec->hi[3]));
}

// Stage a described tile: every existing needed piece (both end pieces of
// the interior rows, the seam rows in full), the x-lower ends and, on the
// last chunk, the x-upper ends, by cp.async; commits one group.
template <int N, int K, bool OPEN, int T = 256>
__host__ __device__ __forceinline__ void xcopies(const XMeta *rec, double *buf, int t)
{
  constexpr int NN = N * N, PW = piece_doubles(N), RS = smem_row_stride(N);
  constexpr int KT = ptile::PSlots<N, T>::KT, SPT = ptile::PSlots<N, T>::SPT;
  const int nk = rec->nk, fl = rec->flags;
  const bool hx = (fl & 1) != 0, vy = (fl & 2) != 0, vz = (fl & 4) != 0;
  const int pcol = present_columns<OPEN>(rec);
#pragma unroll
  for (int jj = 0; jj < SPT; jj++) {
    int j, kq;
    if (!ptile::pslot<N, T>(jj, t, j, kq)) continue;
    int sy, sz, pc;
    ptile::needed_piece<N>(j, sy, sz, pc);
    if (!row_exists<N, OPEN>(sy, sz, vy, vz, pcol)) continue;
    const int s = ptile::col_sel<N>(sy, sz);
    const int es = rec->es[s];
    const double *g = rec->col[s] + (long)kq * es + sz * rec->zs[s] + sy * rec->ys[s] + pc * PW;
    double *sp = buf + (kq * NN + sz * N + sy) * RS + pc * PW;
    for (int k = kq; k < nk; k += KT, g += (long)KT * es, sp += KT * NN * RS) cp_async(sp, g, PW);
  }
  double *locol = buf + K * NN * RS, *hicol = locol + NN;
  for (int r = t; r < NN; r += T) {
    const int sy = r % N, sz = r / N;
    if (!row_exists<N, OPEN>(sy, sz, vy, vz, pcol)) continue;
    const int s = ptile::col_sel<N>(sy, sz);
    const double *lo = rec->lo[s];
    if (!OPEN || lo) cp_async(locol + r, lo + sz * rec->lzs[s] + sy * rec->lys[s], 1);
    if (hx) {
      const double *hi = rec->hi[s];
      if (!OPEN || hi) cp_async(hicol + r, hi + sz * rec->hzs[s] + sy * rec->hys[s], 1);
    }
  }
  cp_commit();
}

// x pairs of every existing row: (element k-1 at n-1, or the lower end)
// with (element k at 0, or, for k = nk on the last chunk, the upper end),
// over the copies that exist.  An interior row (sy, sz in 1..n-2; always
// the rank's own column 0) is final there and stored: point 0 of element k,
// and point n-1 of element k-1 or the lower end where it is the rank's own.
template <int N, int K, bool OPEN, int T = 256>
__host__ __device__ __forceinline__ void xxpass(double *buf, const XMeta *meta, int t)
{
  constexpr int NN = N * N, RS = smem_row_stride(N);
  constexpr long N3 = (long)N * N * N;
  const int nk = meta->nk, fl = meta->flags;
  const bool hx = (fl & 1) != 0, vy = (fl & 2) != 0, vz = (fl & 4) != 0;
  const int pcol = present_columns<OPEN>(meta);
  double *locol = buf + K * NN * RS, *hicol = locol + NN;
  const int items = (nk + (hx ? 1 : 0)) * NN;
  for (int i = t; i < items; i += T) {
    const int k = i / NN, r = i - k * NN;
    const int sy = r % N, sz = r / N;
    if (!row_exists<N, OPEN>(sy, sz, vy, vz, pcol)) continue;
    const int sel = ptile::col_sel<N>(sy, sz);
    const bool pl = !OPEN || k > 0 || meta->lo[sel], ph = !OPEN || k < nk || meta->hi[sel];
    double *lo = k == 0 ? locol + r : buf + ((k - 1) * NN + r) * RS + (N - 1);
    double *hi = k == nk ? hicol + r : buf + (k * NN + r) * RS;
    double s;
    if (!OPEN || (pl && ph)) {
      s = *lo + *hi;
      *lo = s;
      *hi = s;
    } else {
      s = pl ? *lo : *hi;
    }
    if (sy >= 1 && sy <= N - 2 && sz >= 1 && sz <= N - 2) {
      double *g = meta->col[0] + k * N3 + sz * N * N + sy * N;
      if (k < nk) g[0] = s;
      if (k > 0) g[-N3 + (N - 1)] = s;
      else if (meta->wlo & 1) meta->lo[0][sz * N * N + sy * N] = s;
    }
  }
}

// y pairs of rows (0|n-1, o), z pairs of rows (o, 0|n-1) for o in 1..n-2,
// and the corner rows (y, then z), column by column over the tile's points
// and its lower end column, over the rows that exist; each final value is
// stored to the copies that are the rank's own.  The last point of the chunk
// is stored only when the tile takes the upper seam (else the next chunk's
// tile stores it as its lower end); the lower end column is stored only
// where it is the rank's.
template <int N, int K, bool OPEN, int T = 256>
__host__ __device__ __forceinline__ void xyzpass(const double *buf, const XMeta *meta, int t)
{
  constexpr int NN = N * N, RS = smem_row_stride(N);
  constexpr int G = 2 * (N - 2) + 1, COLS = K * N + 1;
  constexpr long N3 = (long)NN * N;
  const int nk = meta->nk, fl = meta->flags;
  const bool hx = (fl & 1) != 0, vy = (fl & 2) != 0, vz = (fl & 4) != 0;
  const double *locol = buf + K * NN * RS;
  const int last_c = (nk - 1) * N + (N - 1);
  const int wcol = meta->wcol, wlo = meta->wlo;
  const int pcol = present_columns<OPEN>(meta), plo = present_lower_ends<OPEN>(meta);
  for (int i = t; i < G * COLS; i += T) {
    const int g = i / COLS, c = i - g * COLS;
    // the group's rows exist?
    if (g < N - 2 ? vz : (g < 2 * (N - 2) ? vy : false)) continue;
    const double *sb;
    int srs, k = 0, x = 0;
    bool lo = false;
    if (c < K * N) {
      k = c / N;
      x = c - k * N;
      if (k >= nk) continue;
      sb = buf + k * NN * RS + x;
      srs = RS;
    } else {
      if (!wlo) continue;
      sb = locol;
      srs = 1;
      lo = true;
    }
    const bool store = lo || hx || c != last_c;
    // the copy of row (sy, sz) at this column exists
    auto present = [&](int sy, int sz) {
      if (!OPEN) return true;
      return ((((lo ? plo : pcol) >> ptile::col_sel<N>(sy, sz)) & 1)) != 0;
    };
    // the rank's own copy of row (sy, sz) at this column, or null
    const long off = lo ? 0 : (long)k * N3 + x;
    auto gaddr = [&](int sy, int sz) -> double * {
      const int sel = ptile::col_sel<N>(sy, sz);
      if (!(((lo ? wlo : wcol) >> sel) & 1)) return nullptr;
      return (lo ? meta->lo[sel] : meta->col[sel]) + off + sz * NN + sy * N;
    };
    if (g < 2 * (N - 2)) {
      int ay, az, by, bz;
      if (g < N - 2) { ay = N - 1; by = 0; az = bz = 1 + g; }      // y pair
      else { ay = by = 1 + g - (N - 2); az = N - 1; bz = 0; }      // z pair
      const bool pa = present(ay, az), pb = present(by, bz);
      if (!pa && !pb) continue;
      const double s = OPEN ? psum(pa ? sb[(az * N + ay) * srs] : 0.0, pa, pb ? sb[(bz * N + by) * srs] : 0.0, pb)
                            : sb[(az * N + ay) * srs] + sb[(bz * N + by) * srs];
      if (store) {
        if (double *p = gaddr(ay, az)) *p = s;
        if (double *p = gaddr(by, bz)) *p = s;
      }
    } else {
      double s;
      if (OPEN) {
        const bool p00 = present(0, 0), p10 = present(N - 1, 0), p01 = present(0, N - 1), p11 = present(N - 1, N - 1);
        if (!(p00 || p10 || p01 || p11)) continue;
        const double c00 = p00 ? sb[0] : 0.0, c10 = p10 ? sb[(N - 1) * srs] : 0.0;
        const double c01 = p01 ? sb[(N - 1) * N * srs] : 0.0, c11 = p11 ? sb[(NN - 1) * srs] : 0.0;
        const double y0 = psum(c10, p10, c00, p00), y1 = psum(c11, p11, c01, p01);
        s = psum(y1, p11 || p01, y0, p10 || p00);
      } else {
        const double c00 = sb[0], c10 = sb[(N - 1) * srs];
        const double c01 = sb[(N - 1) * N * srs], c11 = sb[(NN - 1) * srs];
        const double y0 = c10 + c00, y1 = c11 + c01;
        s = y1 + y0;
      }
      if (store) {
        if (double *p = gaddr(0, 0)) *p = s;
        if (double *p = gaddr(N - 1, 0)) *p = s;
        if (double *p = gaddr(0, N - 1)) *p = s;
        if (double *p = gaddr(N - 1, N - 1)) *p = s;
      }
    }
  }
}

#undef FACES_XLDG

}  // namespace xtile
}  // namespace faces
