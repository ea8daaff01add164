// tile_ops.cuh -- the shared-memory tile step: what each thread copies in,
// sums and copies out.  Host- and device-callable so the CPU replay in
// tests/native runs exactly this code.
//
// A tile is the x-chunk [jx0, jx1) of an element column (rank, jy, jz) with
// the n x n physical rows of rows_setup.cuh (slot (sy,sz) = row (sy,sz) of
// element (jy', jz'), the top rows taken from the elements below).  The tile
// is staged in shared memory, every shared point the tile owns is summed
// ONCE by one thread (x pairs, then y pairs, then z pairs) and written to all
// its staged copies, and the rows go back to global memory.  Compared with
// summing inside each row's thread, each FP64 add is done once and the adds
// of a warp are dense -- GB300's FP64 pipe is narrow, so this matters.
//
// Shared memory of one stage (doubles):
//   buf[k][r][RS]   k < K main elements, r = sy + n*sz, RS >= n (even,
//                   2 mod 4: smem_row_stride)
//   locol[r]        x-lower copy of the first seam (element jx0-1, point n-1)
//   hicol[r]        x-upper copy of the last seam (element mx, point 0)
// and per-row metadata (RowMeta).
#pragma once

#include "geom.cuh"
#include "rows_setup.cuh"

namespace faces {

// flags of a staged row
enum : unsigned {
  kRowValid = 1u,     // the row exists (local or received)
  kRowWritable = 2u,  // local: copied back
  kLoOk = 4u,         // x-lower end exists
  kLoWritable = 8u,
  kHiOk = 16u,        // x-upper end exists (virtual element mx)
  kInterior = 32u,    // sy, sz both in [1, n-2]: only points 0 and n-1 change
};

struct RowMeta {
  const double *rd;  // row of element 0
  const double *lo;
  const double *hi;
  long es;
  unsigned flags;
};

// Row stride of a stage in shared memory: the smallest even stride >= n that
// is 2 mod 4 doubles (16 mod 32 bytes).  Even keeps every row 16-byte
// aligned for the 16-byte copies; 2 mod 4 spreads the rows of a warp's x
// pass (one row per lane, rows RS doubles apart) over 8 of the 16 bank
// pairs, the fewest wavefronts a 64-bit access pattern at that stride
// allows (a stride of 0 mod 8 doubles, e.g. 8 for n = 6, put every row on
// the same banks: 16-way conflicts).
FACES_HD constexpr int smem_row_stride(int n) { return (n + 1) / 2 % 2 == 1 ? (n + 1) / 2 * 2 : (n + 1) / 2 * 2 + 2; }

// piece = the unit of one copy instruction: 2 doubles (16 bytes) for even n,
// 1 double for odd n (rows are then only 8-byte aligned)
FACES_HD constexpr int piece_doubles(int n) { return n % 2 == 0 ? 2 : 1; }
FACES_HD constexpr int pieces_per_row(int n) { return n / piece_doubles(n); }

FACES_HD void row_meta(const FieldDesc &f, const TileCoords &t, int r, RowMeta &m)
{
  const int n = f.n;
  const int sy = r % n, sz = r / n;
  SlotSetup s;
  slot_setup(f, t, sy, sz, n, s);
  m.rd = s.rd;
  m.es = s.es;
  m.lo = s.lo;
  m.hi = t.hi_x ? s.hi : nullptr;
  m.flags = (s.valid ? kRowValid : 0u) | (s.writable ? kRowWritable : 0u) | (s.lo ? kLoOk : 0u) |
            (s.lo && s.lo_w ? kLoWritable : 0u) | (t.hi_x && s.hi ? kHiOk : 0u) |
            ((sy >= 1 && sy <= n - 2 && sz >= 1 && sz <= n - 2) ? kInterior : 0u);
}

// Row metadata for a tile that follows the previous chunk of the same column
// (`follow`, the previous tile's metadata in prev): only the seam ends
// change.  Otherwise the full setup of row_meta.
FACES_HD void tile_row_meta(const FieldDesc &f, const TileCoords &t, bool follow, const RowMeta *prev, int r,
                            RowMeta &m)
{
  const int n = f.n;
  if (!follow) {
    row_meta(f, t, r, m);
    return;
  }
  m = prev[r];
  m.flags &= ~(kLoOk | kLoWritable | kHiOk);
  m.lo = m.hi = nullptr;
  if (m.flags & kRowValid) {
    m.lo = m.rd + (long)(t.jx0 - 1) * m.es + (n - 1);
    m.flags |= kLoOk | ((m.flags & kRowWritable) ? kLoWritable : 0u);
    if (t.hi_x) {
      SlotSetup s;
      slot_setup(f, t, r % n, r / n, n, s);
      m.hi = s.hi;
      if (s.hi) m.flags |= kHiOk;
    }
  }
}

// Per-slot column state: a thread owns the same slots (row r, piece pc) in
// every tile, and a row's source (pointer to its element-0 copy, element
// stride, flags) changes only with the column (rank, jy, jz).
struct SlotCol {
  const double *rd;
  int es;
  unsigned fl;  // kRowValid | kRowWritable | kInterior
};

FACES_HD SlotCol slot_col(const FieldDesc &f, const TileCoords &t, int r)
{
  const int n = f.n, sy = r % n, sz = r / n;
  SlotSetup ss;
  slot_setup(f, t, sy, sz, n, ss);
  SlotCol c;
  c.rd = ss.rd;
  c.es = (int)ss.es;
  c.fl = (ss.valid ? kRowValid : 0u) | (ss.writable ? kRowWritable : 0u) |
         ((sy >= 1 && sy <= n - 2 && sz >= 1 && sz <= n - 2) ? kInterior : 0u);
  return c;
}

// x ends of row r in tile t: inside a column the previous chunk's last point
// (from the column state), at the column's ends the neighbours' (full setup,
// once per column end); returns the row's flags
FACES_HD unsigned row_ends(const FieldDesc &f, const TileCoords &t, const SlotCol &c, int r, const double *&lo,
                           const double *&hi)
{
  const int n = f.n;
  bool lo_w = false;
  lo = hi = nullptr;
  if (t.c > 0 && !t.hi_x) {
    if (c.fl & kRowValid) {
      lo = c.rd + (long)(t.jx0 - 1) * c.es + (n - 1);
      lo_w = (c.fl & kRowWritable) != 0;
    }
  } else {
    SlotSetup ss;
    slot_setup(f, t, r % n, r / n, n, ss);
    lo = ss.lo;
    lo_w = ss.lo && ss.lo_w;
    hi = t.hi_x ? ss.hi : nullptr;
  }
  return c.fl | (lo ? kLoOk : 0u) | (lo_w ? kLoWritable : 0u) | (hi ? kHiOk : 0u);
}

// Copies in and out.  Thread-owned slots (r, p) -- staged row r, piece p --
// repeat over the tile's elements k with fixed strides, so no index is
// divided per copy.  Interior rows move only their first and last piece:
// the step neither reads nor writes their other points.
struct Move {
  const double *g;
  double *s;
  int len;
};

FACES_HD bool piece_needed(int n, unsigned flags, int p)
{
  const int np = pieces_per_row(n);
  return !(flags & kInterior) || p == 0 || p == np - 1;
}

// element k of slot (r, p): global and shared addresses
FACES_HD void slot_move(int n, const RowMeta &m, int r, int p, int jx0, int k, double *buf, Move &mv)
{
  const int pw = piece_doubles(n);
  mv.g = m.rd + (long)(jx0 + k) * m.es + p * pw;
  mv.s = buf + (k * n * n + r) * smem_row_stride(n) + p * pw;
  mv.len = pw;
}

// Copy-out of slot (r, p) element k: the last element's point n-1 belongs to
// the next chunk's first seam unless this tile takes the extra seam step
// (hi_x).  Returns the doubles to store (0: none).
FACES_HD int slot_out_len(int n, int nk, bool hi_x, int p, int k)
{
  const int np = pieces_per_row(n), pw = piece_doubles(n);
  return (k == nk - 1 && !hi_x && p == np - 1) ? pw - 1 : pw;
}

// Groups of a tile with nk main elements: the shared points whose canonical
// copy (index 0 on every seam axis, else in [1, n-2]) lies in the tile.
// Enumerated class by class across the tile's elements so that a warp's
// threads take the same code path: the x, y, z faces ((n-2)^2 each per
// element), the edges along z, y, x (n-2 each: xy, xz, yz seams), the
// corners; then, with hi_x, the seam with element mx (a virtual element nk
// with ix = 0: its x face, xy and xz edges and corner).
FACES_HD int classes_size(int n, int cls)
{
  const int ni = n - 2;
  return cls < 3 ? ni * ni : cls < 6 ? ni : 1;
}

FACES_HD long tile_groups(int n, int nk, bool hi_x)
{
  const long ni = n - 2;
  return (long)nk * (3 * ni * ni + 3 * ni + 1) + (hi_x ? ni * ni + 2 * ni + 1 : 0);
}

// group g -> element k and point (ix, iy, iz)
FACES_HD void group_point(int n, int nk, long g, int &k, int &ix, int &iy, int &iz)
{
  const int ni = n - 2;
  int q = (int)g;
  // main elements: class-major
  for (int cls = 0; cls < 7; cls++) {
    const int c = classes_size(n, cls);
    if (q < nk * c) {
      k = q / c;
      const int j = q - k * c;
      const int a = 1 + j % (ni > 0 ? ni : 1), b = 1 + j / (ni > 0 ? ni : 1);
      switch (cls) {
        case 0: ix = 0; iy = a; iz = b; break;   // x face
        case 1: ix = a; iy = 0; iz = b; break;   // y face
        case 2: ix = a; iy = b; iz = 0; break;   // z face
        case 3: ix = 0; iy = 0; iz = 1 + j; break;  // xy edge (along z)
        case 4: ix = 0; iy = 1 + j; iz = 0; break;  // xz edge (along y)
        case 5: ix = 1 + j; iy = 0; iz = 0; break;  // yz edge (along x)
        default: ix = 0; iy = 0; iz = 0; break;     // corner
      }
      return;
    }
    q -= nk * c;
  }
  // virtual element nk (ix = 0)
  k = nk;
  ix = 0;
  if (q < ni * ni) { iy = 1 + q % ni; iz = 1 + q / ni; return; }
  q -= ni * ni;
  if (q < ni) { iy = 0; iz = 1 + q; return; }
  q -= ni;
  if (q < ni) { iy = 1 + q; iz = 0; return; }
  iy = 0; iz = 0;
}

// The copies of one group along x for staged row r: the upper copy (element
// k at ix, or the received x-upper end for the virtual element) and, on an x
// seam, the lower copy (element k-1 at n-1, or the x-lower end for k = 0).
template <bool SX>
FACES_HD void x_level(int n, int nk, const unsigned *rflags, double *buf, double *locol, double *hicol, int k, int ix,
                      int r, double *&pu, bool &ou, double *&pl, bool &ol, double &v, bool &present, int &cnt)
{
  const int NN = n * n, RS = smem_row_stride(n);
  const unsigned fl = rflags[r];
  if (k == nk) { pu = hicol + r; ou = (fl & kHiOk) != 0; }
  else { pu = buf + (k * NN + r) * RS + ix; ou = (fl & kRowValid) != 0; }
  double vu = ou ? *pu : 0.0;
  if (SX) {
    if (k == 0) { pl = locol + r; ol = (fl & kLoOk) != 0; }
    else { pl = buf + ((k - 1) * NN + r) * RS + (n - 1); ol = (fl & kRowValid) != 0; }
    const double vl = ol ? *pl : 0.0;
    v = ol ? (ou ? vl + vu : vl) : vu;
    cnt += (int)ol + (int)ou;
  } else {
    pl = nullptr;
    ol = false;
    v = vu;
    cnt += (int)ou;
  }
  present = ou || ol;
}

// sum of one group: x pairs, then y pairs, then z pairs over the copies that
// exist, written to every staged copy
template <bool SX, bool SY, bool SZ>
FACES_HD void group_sum(int n, int nk, const unsigned *rflags, double *buf, double *locol, double *hicol, int k, int ix,
                        int iy, int iz)
{
  double *pu[2][2], *pl[2][2];
  bool ou[2][2], ol[2][2], pr[2][2];
  double v[2][2];
  int cnt = 0;
#pragma unroll
  for (int bz = 0; bz < 2; bz++)
#pragma unroll
    for (int by = 0; by < 2; by++) {
      pr[bz][by] = false;
      v[bz][by] = 0.0;
      ou[bz][by] = ol[bz][by] = false;
      pu[bz][by] = pl[bz][by] = nullptr;
      if ((!SY && by == 0) || (!SZ && bz == 0)) continue;
      const int r = (by ? iy : n - 1) + n * (bz ? iz : n - 1);
      x_level<SX>(n, nk, rflags, buf, locol, hicol, k, ix, r, pu[bz][by], ou[bz][by], pl[bz][by], ol[bz][by],
                  v[bz][by], pr[bz][by], cnt);
    }
  if (cnt < 2) return;
  double w[2];
  bool pw[2];
#pragma unroll
  for (int bz = 0; bz < 2; bz++) {
    if (SY) w[bz] = pr[bz][0] ? (pr[bz][1] ? v[bz][0] + v[bz][1] : v[bz][0]) : v[bz][1];
    else w[bz] = v[bz][1];
    pw[bz] = pr[bz][0] || pr[bz][1];
  }
  const double s = SZ ? (pw[0] ? (pw[1] ? w[0] + w[1] : w[0]) : w[1]) : w[1];
#pragma unroll
  for (int bz = 0; bz < 2; bz++)
#pragma unroll
    for (int by = 0; by < 2; by++) {
      if (ou[bz][by]) *pu[bz][by] = s;
      if (SX && ol[bz][by]) *pl[bz][by] = s;
    }
}

FACES_HD void tile_group_at(int n, int nk, const unsigned *rflags, double *buf, double *locol, double *hicol, int k,
                            int ix, int iy, int iz)
{
  const int pat = (ix == 0 ? 1 : 0) | (iy == 0 ? 2 : 0) | (iz == 0 ? 4 : 0);
  switch (pat) {
    case 1: group_sum<true, false, false>(n, nk, rflags, buf, locol, hicol, k, ix, iy, iz); break;
    case 2: group_sum<false, true, false>(n, nk, rflags, buf, locol, hicol, k, ix, iy, iz); break;
    case 4: group_sum<false, false, true>(n, nk, rflags, buf, locol, hicol, k, ix, iy, iz); break;
    case 3: group_sum<true, true, false>(n, nk, rflags, buf, locol, hicol, k, ix, iy, iz); break;
    case 5: group_sum<true, false, true>(n, nk, rflags, buf, locol, hicol, k, ix, iy, iz); break;
    case 6: group_sum<false, true, true>(n, nk, rflags, buf, locol, hicol, k, ix, iy, iz); break;
    case 7: group_sum<true, true, true>(n, nk, rflags, buf, locol, hicol, k, ix, iy, iz); break;
    default: break;
  }
}

FACES_HD void tile_group(int n, int nk, const unsigned *rflags, double *buf, double *locol, double *hicol, long g)
{
  int k, ix, iy, iz;
  group_point(n, nk, g, k, ix, iy, iz);
  tile_group_at(n, nk, rflags, buf, locol, hicol, k, ix, iy, iz);
}

struct TileSmemLayout {
  long buf, locol, hicol, meta_bytes_off;  // offsets in doubles; meta after
  long doubles;                            // per stage, data part
};

// Elements per tile by default: as many as fit a ~20 KB stage, rounded down
// to a power of 2 in [1, 32] (three stages and three resident blocks per SM
// then fit in shared memory).
FACES_HD constexpr int tile_kmax(int n)
{
  return 20480 / (n * n * smem_row_stride(n) * 8) >= 32 ? 32
         : 20480 / (n * n * smem_row_stride(n) * 8) >= 16 ? 16
         : 20480 / (n * n * smem_row_stride(n) * 8) >= 8  ? 8
         : 20480 / (n * n * smem_row_stride(n) * 8) >= 4  ? 4
         : 20480 / (n * n * smem_row_stride(n) * 8) >= 2  ? 2
                                                           : 1;
}

// Elements per tile of the warp-tile form (one warp per tile): as many as
// fit a ~6 KB stage, a power of 2 in [1, 32].
FACES_HD constexpr int tile_kwarp(int n)
{
  return 6144 / (n * n * smem_row_stride(n) * 8) >= 32 ? 32
         : 6144 / (n * n * smem_row_stride(n) * 8) >= 16 ? 16
         : 6144 / (n * n * smem_row_stride(n) * 8) >= 8  ? 8
         : 6144 / (n * n * smem_row_stride(n) * 8) >= 4  ? 4
         : 6144 / (n * n * smem_row_stride(n) * 8) >= 2  ? 2
                                                          : 1;
}

// the kernel is instantiated for K = 1, 2, 4, ..., tile_kinst_max(n)
// elements per tile; a plan whose chunk is smaller (clamped to mx) runs in
// the next larger instance
FACES_HD constexpr int tile_kinst_max(int n) { return tile_kmax(n) > 8 ? tile_kmax(n) : 8; }
FACES_HD int tile_instance_k(int chunk)
{
  return chunk <= 1 ? 1 : chunk <= 2 ? 2 : chunk <= 4 ? 4 : chunk <= 8 ? 8 : chunk <= 16 ? 16 : 32;
}

FACES_HD long tile_stage_doubles(int n, int K)
{
  return (long)K * n * n * smem_row_stride(n) + 2L * n * n;
}

}  // namespace faces

namespace faces {

// ---------------------------------------------------------------------------
// Regular tiles (every staged row present, both x ends present where needed
// -- every tile of a periodic field): the sums are three dense passes over
// the staged rows, the in-place passes of the reference's Mugs oracle
// (gpu/Mugs.cc:140-202) restricted to one tile: x pairs, then y pairs, then
// z pairs.  Each item reads two staged cells, adds once, writes both; the
// items of one pass touch disjoint cells.  The two copies of an x-seam point
// (element k-1 at n-1, element k at 0) hold equal values after the x pass,
// so the y and z passes may sum both.
// ---------------------------------------------------------------------------

// a tile whose every row and needed x end is present takes the passes
FACES_HD bool row_regular(unsigned flags, bool hi_x)
{
  return (flags & kRowValid) && (flags & kLoOk) && (!hi_x || (flags & kHiOk));
}

// x pass: item (k, r), k in [0, nk] (k = nk only with hi_x): the seam
// between element k-1 (or the lower end) and element k (or the upper end)
FACES_HD int xpass_items(int n, int nk, bool hi_x) { return (nk + (hi_x ? 1 : 0)) * n * n; }

FACES_HD void xpass_at(int n, int nk, double *buf, double *locol, double *hicol, int k, int r)
{
  const int NN = n * n, RS = smem_row_stride(n);
  double *lo = k == 0 ? locol + r : buf + ((k - 1) * NN + r) * RS + (n - 1);
  double *hi = k == nk ? hicol + r : buf + (k * NN + r) * RS;
  const double s = *lo + *hi;
  *lo = s;
  *hi = s;
}

FACES_HD void xpass_item(int n, int nk, double *buf, double *locol, double *hicol, int i)
{
  xpass_at(n, nk, buf, locol, hicol, i / (n * n), i % (n * n));
}

// y pass (axis 1) and z pass (axis 2): item (o, c) pairs the lower row
// (index n-1 on the axis) with the upper row (index 0) -- o is the row index
// on the other axis -- at staged column c: c < nk*n is point c%n of element
// c/n, c = nk*n the lower end column, c = nk*n+1 the upper end column (with
// hi_x only)
FACES_HD int yz_span(int n, int nk, bool hi_x) { return nk * n + 1 + (hi_x ? 1 : 0); }
FACES_HD int yzpass_items(int n, int nk, bool hi_x) { return n * yz_span(n, nk, hi_x); }

FACES_HD void yzpass_at(int n, int nk, int axis, double *buf, double *locol, double *hicol, int o, int c)
{
  const int NN = n * n, RS = smem_row_stride(n);
  const int r_lo = axis == 1 ? (n - 1) + n * o : o + n * (n - 1);
  const int r_hi = axis == 1 ? n * o : o;
  double *a, *b;
  if (c < nk * n) {
    const int k = c / n, x = c - k * n;
    a = buf + (k * NN + r_lo) * RS + x;
    b = buf + (k * NN + r_hi) * RS + x;
  } else if (c == nk * n) {
    a = locol + r_lo;
    b = locol + r_hi;
  } else {
    a = hicol + r_lo;
    b = hicol + r_hi;
  }
  const double s = *a + *b;
  *a = s;
  *b = s;
}

FACES_HD void yzpass_item(int n, int nk, bool hi_x, int axis, double *buf, double *locol, double *hicol, int i)
{
  const int span = yz_span(n, nk, hi_x);
  yzpass_at(n, nk, axis, buf, locol, hicol, i / span, i % span);
}

}  // namespace faces
