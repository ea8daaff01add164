// rows_setup.cuh -- where each thread of the row kernel reads and writes.
//
// Host- and device-callable, so the same code that the kernel runs can be
// replayed on the CPU to check every address against its buffer and that no
// field point is written twice in one share (tests/native/rows_plan_check.cc).
//
// Tiles.  A tile is one x-chunk [jx0, jx1) of an element column (rank r, jy,
// jz).  It owns the shared points whose rank-local coordinates lie in
// [jx0*(n-1), jx1*(n-1)) x [jy*(n-1), (jy+1)*(n-1)) x [jz*(n-1), (jz+1)*(n-1)).
// Their copies sit in exactly n x n physical rows: slot (sy, sz) reads row
// (iy, iz) = (sy, sz) of element (jy', jz') with jy' = jy for sy < n-1 and
// jy-1 for sy = n-1 (likewise z) -- the lower element's top row holds the
// other copy of the points in row 0.  Every element row of the field belongs
// to exactly one slot of one tile, so each row is read once and written once
// per share and no two threads touch the same point.
//
// Ranks.  jy-1 = -1 is the lower neighbour rank's top element: its memory in
// direct mode, its message in message mode.  In message mode, or at a
// non-periodic top, the column also gets a virtual top tile jy = my whose row
// 0 is the upper neighbour's message (or absent) and whose row n-1 is the top
// element's; likewise along x the last chunk takes one more step, to the
// seam with element mx.
#pragma once

#include "geom.cuh"

namespace faces {

struct RowPlan {
  int chunk;      // elements per x-chunk (K)
  int nchunks;    // ceil(mx / K)
  int ty, tz;     // tile rows in y and z (m, or m+1 with a virtual top tile)
  long ntiles;    // nranks * tz * ty * nchunks
  int tiles_per_block;
  int order;      // tile kernel: 0 grid-stride over tiles, 1 contiguous range per
                  // block, 2 grid-stride over units of unit_chunks chunks of a column
  int unit_chunks;
};

FACES_HD int nbr_of(const FieldDesc &f, int r, int dir) { return f.nbr[r * 27 + dir]; }

// the message rank r receives from direction dir: what neighbour(r,dir) sent
// toward the opposite direction (26-dir)
FACES_HD const double *recv_of(const FieldDesc &f, int r, int dir)
{
  const int q = f.nbr[r * 27 + dir];
  if (q < 0) return nullptr;
  return f.msg + f.msg_off[q * 27 + (26 - dir)];
}

FACES_HD constexpr int pow2_at_least(int n) { return n <= 2 ? 2 : n <= 4 ? 4 : n <= 8 ? 8 : 16; }
// threads of one tile: P = pow2_at_least(n) slots per y-row keep the y pairs
// of a row inside one warp; the tile is padded to whole warps
FACES_HD constexpr int tile_threads(int n) { return ((pow2_at_least(n) * n + 31) / 32) * 32; }

// the y (axis 1) or z (axis 2) part of slot s in tile row jt: element e of the
// rank offset d along the axis, point index i; false if the copy is absent
FACES_HD bool slot_part(const FieldDesc &f, int r, int axis, int jt, int s, int n, int &e, int &i, int &d)
{
  const int m = f.m[axis];
  int dv[3] = {0, 0, 0};
  if (s < n - 1) {
    if (jt < m) { e = jt; i = s; d = 0; return true; }
    // virtual top tile: row 0 is the upper neighbour's element 0 (messages)
    if (s != 0 || f.mode != kMessages) return false;
    dv[axis] = 1;
    if (nbr_of(f, r, dir_index(dv[0], dv[1], dv[2])) < 0) return false;
    e = 0; i = 0; d = 1;
    return true;
  }
  if (jt >= 1) { e = jt - 1; i = n - 1; d = 0; return true; }
  dv[axis] = -1;
  if (nbr_of(f, r, dir_index(dv[0], dv[1], dv[2])) < 0) return false;
  e = m - 1; i = n - 1; d = -1;
  return true;
}

FACES_HD bool slot_valid(const FieldDesc &f, int r, int jy, int jz, int sy, int sz, int n)
{
  int e, i, d;
  return slot_part(f, r, 1, jy, sy, n, e, i, d) && slot_part(f, r, 2, jz, sz, n, e, i, d);
}

// single value at an x end of a row that lies in the x-neighbour (dx = -1:
// element mx-1, point n-1; dx = +1: element 0, point 0).  Direct mode: a
// pointer into the neighbour rank's memory; message mode: into the message.
FACES_HD const double *x_end(const FieldDesc &f, int r, int dx, int dy, int dz, int iy, int iz, int ey, int ez,
                             bool &writable)
{
  const int dir = dir_index(dx, dy, dz);
  const int q = nbr_of(f, r, dir);
  writable = false;
  if (q < 0) return nullptr;
  const int n = f.n;
  if (f.mode == kDirect) {
    writable = true;
    const int ix = dx < 0 ? n - 1 : 0, jx = dx < 0 ? f.m[0] - 1 : 0;
    return f.u + (long)q * f.R + elem_index(f, ix, iy, iz, jx, ey, ez);
  }
  const int d[3] = {dx, dy, dz};
  const int i[3] = {0, iy, iz}, j[3] = {0, ey, ez};
  return recv_of(f, r, dir) + region_pos(f, d, i, j);
}

FACES_HD RowPlan make_row_plan(const FieldDesc &f, int chunk, int tiles_per_block)
{
  RowPlan p;
  p.chunk = chunk < 1 ? 1 : (chunk > f.m[0] ? f.m[0] : chunk);
  p.nchunks = (f.m[0] + p.chunk - 1) / p.chunk;
  const bool virt = f.mode == kMessages || !f.periodic;
  p.ty = f.m[1] + (virt ? 1 : 0);
  p.tz = f.m[2] + (virt ? 1 : 0);
  p.ntiles = (long)f.nranks * p.tz * p.ty * p.nchunks;
  const int tt = tile_threads(f.n);
  int tpb = tiles_per_block > 0 ? tiles_per_block : 256 / tt;
  if (tpb < 1) tpb = 1;
  if (tpb * tt > 256) tpb = 256 / tt;
  if (tpb > 15) tpb = 15;  // named barriers 1..15
  p.tiles_per_block = tpb;
  p.order = 0;
  p.unit_chunks = 1;
  return p;
}

// A tile whose rows are all local, with its x-lower end in the same column and
// no x-upper end: not the first or last chunk of its column, not the first or
// a virtual top row of elements in y or z.  The periodic step handles these
// tiles of any field exactly as the general step does.
FACES_HD bool interior_tile(const FieldDesc &f, int nchunks, int c, int jy, int jz)
{
  return c >= 1 && c < nchunks - 1 && jy >= 1 && jy < f.m[1] && jz >= 1 && jz < f.m[2];
}

struct TileCoords {
  int r, jy, jz, c;
  int jx0, jx1;
  bool skip;  // virtual top tile this rank does not need
  bool hi_x;  // last chunk takes the extra seam step with element mx
};

// Mixed-radix position of a tile, (chunk, jy, jz, rank) with radices
// (nchunks, ty, tz, nranks): a block walks its tiles by adding a constant
// step to a cursor, without dividing per tile.
struct TileCursor {
  int c, jy, jz, r;
};

FACES_HD TileCursor cursor_of(const RowPlan &p, long tile)
{
  TileCursor u;
  long q = tile;
  u.c = (int)(q % p.nchunks); q /= p.nchunks;
  u.jy = (int)(q % p.ty); q /= p.ty;
  u.jz = (int)(q % p.tz); q /= p.tz;
  u.r = (int)q;
  return u;
}

FACES_HD void cursor_add(const RowPlan &p, TileCursor &a, const TileCursor &d)
{
  a.c += d.c;
  int carry = a.c >= p.nchunks;
  if (carry) a.c -= p.nchunks;
  a.jy += d.jy + carry;
  carry = a.jy >= p.ty;
  if (carry) a.jy -= p.ty;
  a.jz += d.jz + carry;
  carry = a.jz >= p.tz;
  if (carry) a.jz -= p.tz;
  a.r += d.r + carry;
}

FACES_HD TileCoords coords_of(const FieldDesc &f, const RowPlan &p, const TileCursor &u)
{
  TileCoords t;
  t.c = u.c;
  t.jy = u.jy;
  t.jz = u.jz;
  t.r = u.r;
  t.jx0 = t.c * p.chunk;
  t.jx1 = t.jx0 + p.chunk < f.m[0] ? t.jx0 + p.chunk : f.m[0];
  // direct mode: a virtual top tile exists only where no upper rank owns the
  // shared plane (non-periodic top)
  t.skip = (t.jy == f.m[1] && f.mode != kMessages && nbr_of(f, t.r, dir_index(0, 1, 0)) >= 0) ||
           (t.jz == f.m[2] && f.mode != kMessages && nbr_of(f, t.r, dir_index(0, 0, 1)) >= 0);
  t.hi_x = (t.c == p.nchunks - 1) && (f.mode == kMessages || nbr_of(f, t.r, dir_index(1, 0, 0)) < 0);
  return t;
}

FACES_HD TileCoords tile_coords(const FieldDesc &f, const RowPlan &p, long tile)
{
  return coords_of(f, p, cursor_of(p, tile));
}

struct SlotSetup {
  bool active, valid, writable;
  const double *rd;  // the row of element 0 (rd + jx*es is element jx's row)
  long es;
  int ey, ez, iy, iz, dy, dz;
  bool yseam, zseam;
  bool pvy, pvz, pvyz;  // partner rows exist: y, z, and z's y partner
  // x-lower end of the first seam of the chunk (element jx0-1, point n-1)
  const double *lo;
  bool lo_w;
  // x-upper end of the last chunk's extra seam (element mx, point 0)
  const double *hi;
};

FACES_HD void slot_setup(const FieldDesc &f, const TileCoords &t, int sy, int sz, int P, SlotSetup &s)
{
  const int n = f.n, mx = f.m[0];
  s.active = sy < n && sz < n;
  s.valid = s.writable = false;
  s.rd = nullptr;
  s.es = 0;
  s.ey = s.ez = s.iy = s.iz = s.dy = s.dz = 0;
  s.lo = s.hi = nullptr;
  s.lo_w = false;
  (void)P;
  if (s.active) {
    const bool vy = slot_part(f, t.r, 1, t.jy, sy, n, s.ey, s.iy, s.dy);
    const bool vz = slot_part(f, t.r, 2, t.jz, sz, n, s.ez, s.iz, s.dz);
    s.valid = vy && vz;
    if (s.valid) {
      if ((s.dy == 0 && s.dz == 0) || f.mode == kDirect) {
        const int q = (s.dy == 0 && s.dz == 0) ? t.r : nbr_of(f, t.r, dir_index(0, s.dy, s.dz));
        s.rd = f.u + (long)q * f.R + elem_index(f, 0, s.iy, s.iz, 0, s.ey, s.ez);
        s.es = (long)n * n * n;
        s.writable = true;
      } else {
        // a remote row: the message from direction (0,dy,dz); its free
        // coordinates are x and whichever of y, z is local
        const double *rb = recv_of(f, t.r, dir_index(0, s.dy, s.dz));
        if (s.dy != 0 && s.dz != 0) { s.rd = rb; s.es = n; }
        else if (s.dy != 0) { s.rd = rb + (long)n * s.iz + (long)n * n * mx * s.ez; s.es = (long)n * n; }
        else { s.rd = rb + (long)n * s.iy + (long)n * n * mx * s.ey; s.es = (long)n * n; }
      }
    }
  }
  s.yseam = s.active && (sy == 0 || sy == n - 1);
  s.zseam = s.active && (sz == 0 || sz == n - 1);
  const int syp = (sy == 0) ? n - 1 : 0, szp = (sz == 0) ? n - 1 : 0;
  s.pvy = s.yseam && slot_valid(f, t.r, t.jy, t.jz, syp, sz, n);
  s.pvz = s.zseam && slot_valid(f, t.r, t.jy, t.jz, sy, szp, n);
  s.pvyz = s.zseam && s.yseam && slot_valid(f, t.r, t.jy, t.jz, syp, szp, n);
  if (s.valid) {
    if (t.c > 0) {
      s.lo = s.rd + (long)(t.jx0 - 1) * s.es + (n - 1);
      s.lo_w = s.writable;
    } else {
      bool wr;
      s.lo = x_end(f, t.r, -1, s.dy, s.dz, s.iy, s.iz, s.ey, s.ez, wr);
      s.lo_w = s.lo && wr;
    }
    if (t.hi_x) {
      bool wr;
      // direct mode takes the extra step only without an upper neighbour,
      // so there this is null
      s.hi = x_end(f, t.r, 1, s.dy, s.dz, s.iy, s.iz, s.ey, s.ez, wr);
    }
  }
}

}  // namespace faces
