// v6_steps.cuh -- the v-6 strategy's geometry and the bodies of its kernels
// (host- and device-callable, so that tests/native/ptile_emu.cu replays them
// on the CPU).
//
// v-6 (gpu/v-6-messages-basic/Faces.cc:65-173): six face messages per rank
// and three dimension sweeps, z then y then x.  Face d of a rank holds the
// n*n*m_a*m_b points of its low (i_d = 0, j_d = 0) or high (i_d = n-1,
// j_d = m_d-1) plane, a < b the other two dimensions, point (ia, ib, ja, jb)
// at ia + n*ib + n^2*ja + n^2*m_a*jb (the layout of zfs(ix,iy,jx,jy),
// yfs(ix,iz,jx,jz), xfs(iy,iz,jy,jz)).  Per rank the buffer holds the x, y, z
// faces, low then high.
//
// A sweep runs a thread per independent part (v6_part_at): an element and a
// point of its face across d, summing the element pair along d there (and
// the face message adds at the first and last elements).
//
// The fused form (v-6 overlap-fusable, gpu/v-6-messages-overlap-fusable/
// Faces.cc:65-352, there to overlap the MPI transfers with the sweeps): a
// sweep's part thread finishes the points it touches, so it can pack the
// next sweeps' messages for them as soon as its own update is done, and
// points that no later sweep changes can be packed before the first one.
// Four launches per share instead of six:
//   A  every z face; the y-face points with iz interior; the x-face points
//      with iy and iz interior (no sweep before theirs changes them);
//   B  the z sweep; a part on a y face packs its points (iz on a seam), one
//      on an x face with iy interior packs its points;
//   C  the y sweep; a part on an x face packs its points (iy on a seam);
//   D  the x sweep.
// Every message point is packed exactly once, after the last sweep before
// its own changed it, so the messages and the sums are those of the basic
// form bit for bit.
#pragma once

#include "geom.cuh"
#include "rows_setup.cuh"

namespace faces {

// Dimension d's sweep: a and b are the other two axes (a < b); sp* and se*
// are the point and element strides of each axis, set on the host so that the
// kernels index no array by a run-time axis (that would put it in local
// memory).
struct V6Geom {
  int d, n, ma, mb, md;
  long F, per_rank, off;  // face doubles, doubles per rank, offset of dimension d
  long spa, spb, spd, sea, seb, sed;
};

inline V6Geom v6_geom(const FieldDesc &f, int d)
{
  V6Geom g;
  g.d = d;
  g.n = f.n;
  const int a = d == 0 ? 1 : 0, b = d == 2 ? 1 : 2;
  const long n = f.n, nn = n * n;
  const long sp[3] = {1, n, nn}, se[3] = {nn * n, f.sjy, f.sjz};
  g.ma = f.m[a];
  g.mb = f.m[b];
  g.md = f.m[d];
  g.spa = sp[a];
  g.spb = sp[b];
  g.spd = sp[d];
  g.sea = se[a];
  g.seb = se[b];
  g.sed = se[d];
  const long Fd[3] = {nn * f.m[1] * f.m[2], nn * f.m[0] * f.m[2], nn * f.m[0] * f.m[1]};
  g.F = Fd[d];
  g.per_rank = 2 * (Fd[0] + Fd[1] + Fd[2]);
  g.off = 2 * (d > 0 ? Fd[0] : 0) + 2 * (d > 1 ? Fd[1] : 0);
  return g;
}

// the three sweeps' geometries (index = d)
struct V6Geoms {
  V6Geom g[3];
};

inline V6Geoms v6_geoms(const FieldDesc &f)
{
  V6Geoms s;
  for (int d = 0; d < 3; d++) s.g[d] = v6_geom(f, d);
  return s;
}

// face point idx of a dimension-d face: (ia, ib) fastest, then ja, then jb
struct V6Point {
  int ia, ib, ja, jb;
  long off;  // ia*spa + ib*spb + ja*sea + jb*seb
};

template <typename I>
FACES_HD V6Point v6_point(const V6Geom &g, I idx)
{
  const I n = (I)g.n, nn = n * n, pa = nn * (I)g.ma;
  V6Point p;
  const I jb = idx / pa;
  I q = idx - jb * pa;
  const I ja = q / nn;
  q -= ja * nn;
  const I ib = q / n;
  p.ia = (int)(q - ib * n);
  p.ib = (int)ib;
  p.ja = (int)ja;
  p.jb = (int)jb;
  p.off = p.ia * g.spa + p.ib * g.spb + p.ja * g.sea + p.jb * g.seb;
  return p;
}

// the position of point (ia, ib, ja, jb) in a dimension-g.d face
FACES_HD long v6_face_index(const V6Geom &g, int ia, int ib, int ja, int jb)
{
  const long n = g.n;
  return ia + n * ib + n * n * ja + n * n * g.ma * jb;
}

// the doubles of point (ia, ib, ja, jb) on side `side` of a dimension-g.d
// face, from the rank's field ur (rank r's base)
FACES_HD long v6_face_source(const V6Geom &g, const V6Point &p, int side)
{
  return p.off + (side ? (long)(g.n - 1) * g.spd + (long)(g.md - 1) * g.sed : 0);
}

// basic pack: thread t of nranks*2F -> one point of one side of every rank's
// dimension-g.d faces
template <typename I>
FACES_HD void v6_pack_item(const FieldDesc &f, const V6Geom &g, double *msg, I t)
{
  const I F2 = 2 * (I)g.F;
  const I r = t / F2;
  const I rem = t - r * F2;
  const int side = rem >= (I)g.F;
  const I idx = rem - (side ? (I)g.F : 0);
  const V6Point p = v6_point(g, idx);
  msg[(long)r * g.per_rank + g.off + (side ? g.F : 0) + (long)idx] = f.u[(long)r * f.R + v6_face_source(g, p, side)];
}

// fused launch A: thread t of nranks*per_rank -> message position t (rank,
// then x, y, z faces, low then high); packs the points no sweep before
// theirs changes: z faces whole, y faces with iz interior, x faces with iy
// and iz interior
template <typename I>
FACES_HD void v6_early_item(const FieldDesc &f, const V6Geoms &gs, double *msg, I t)
{
  const long pr = gs.g[0].per_rank;
  const I r = t / (I)pr;
  long rem = (long)(t - r * (I)pr);
  int d = 0;
  while (d < 2 && rem >= 2 * gs.g[d].F) {
    rem -= 2 * gs.g[d].F;
    d++;
  }
  const V6Geom &g = gs.g[d];
  const int side = rem >= g.F;
  const long idx = rem - (side ? g.F : 0);
  const V6Point p = v6_point(g, idx);
  const int n = g.n;
  // dimension 1: b is z; dimension 0: a is y, b is z
  if (d == 1 && (p.ib == 0 || p.ib == n - 1)) return;
  if (d == 0 && (p.ia == 0 || p.ia == n - 1 || p.ib == 0 || p.ib == n - 1)) return;
  msg[(long)r * pr + g.off + (side ? g.F : 0) + idx] = f.u[(long)r * f.R + v6_face_source(g, p, side)];
}

// One sweep (dimension g.d) split over its independent parts, in memory
// order: thread t of nranks * elements * n^2 -> rank, element (jx fastest,
// then jy, jz) and point (ia, ib) of its face across d (fastest).  The thread
// sums the element pair (jd, jd+1) along d at that point, and also the low
// face's add of the lower neighbour's high face when jd = 0 and the high
// face's add of the upper neighbour's low face when jd = md-1: points no
// other thread touches, so the column sweep's sums come out with no chain of
// dependent loads along a column, and concurrent warps work on neighbouring
// elements (the thread layout of gpu/v-6-messages-basic/Faces.cc:48-104,
// one block per element there).
// the part of element (jx, jy, jz) of rank r at face point `face` (ia
// fastest); N = n when known at compile time, else 0
template <int N>
FACES_HD void v6_part_at(const FieldDesc &f, const V6Geom &g, const double *msg, int compute, int r, int jx, int jy,
                         int jz, int face)
{
  const int n = N > 0 ? N : g.n, d = g.d;
  const int ia = face % n, ib = face / n;
  // the element's coordinates along a, b (the face's axes) and d
  const int ja = d == 0 ? jy : jx, jb = d == 2 ? jy : jz, jd = d == 0 ? jx : d == 1 ? jy : jz;
  const long idx = v6_face_index(g, ia, ib, ja, jb);
  const long off = ia * g.spa + ib * g.spb + ja * g.sea + jb * g.seb;
  double *ur = f.u + (long)r * f.R + off;  // this point at coordinate 0 along d, element 0 along d
  const long top = (long)(n - 1) * g.spd;   // i_d = n - 1 within an element
  if (jd == 0) {
    const int lo = nbr_of(f, (int)r, dir_index(d == 0 ? -1 : 0, d == 1 ? -1 : 0, d == 2 ? -1 : 0));
    if (lo >= 0) *ur = *ur + msg[(long)lo * g.per_rank + g.off + g.F + idx];
  }
  if (jd == g.md - 1) {
    const int hi = nbr_of(f, (int)r, dir_index(d == 0 ? 1 : 0, d == 1 ? 1 : 0, d == 2 ? 1 : 0));
    if (hi >= 0) {
      double *p = ur + top + (long)(g.md - 1) * g.sed;
      *p = *p + msg[(long)hi * g.per_rank + g.off + idx];
    }
  } else {
    const bool on_a = (ia == 0 && ja == 0) || (ia == n - 1 && ja == g.ma - 1);
    const bool on_b = (ib == 0 && jb == 0) || (ib == n - 1 && jb == g.mb - 1);
    if (!(compute || on_a || on_b)) return;
    double *p = ur + top + (long)jd * g.sed;
    double *pq = p + g.sed - top;
    const double v = *p + *pq;
    *p = v;
    *pq = v;
  }
}

// Fused launches B (d = 2) and C (d = 1) in the part layout: v6_part_at's
// update, then the messages of the later sweeps for the points it touched --
// every point with i_d in {0, n-1} belongs to exactly one part: (jd, n-1) to
// element jd's pair or high add, (jd, 0) to element jd-1's pair or, for
// jd = 0, the low add.  The z sweep packs a point into the y faces where it
// lies on one (iy = 0 of jy = 0, iy = n-1 of jy = my-1), and into the x
// faces where it lies on one with iy interior (the y sweep packs those with
// iy on a seam); the y sweep packs into the x faces.  The update reads
// dimension d's faces and the packs write the other dimensions'.
template <int N>
FACES_HD void v6_part_pack_at(const FieldDesc &f, const V6Geoms &gs, int d, double *msg, int compute, int r, int jx,
                              int jy, int jz, int face)
{
  const V6Geom &g = gs.g[d];
  v6_part_at<N>(f, g, msg, compute, r, jx, jy, jz, face);
  const int n = N > 0 ? N : g.n, nz = n - 1;
  const int ia = face % n, ib = face / n;
  const int ja = d == 0 ? jy : jx, jb = d == 2 ? jy : jz, jd = d == 0 ? jx : d == 1 ? jy : jz;
  const double *ur = f.u + (long)r * f.R + ia * g.spa + ib * g.spb + ja * g.sea + jb * g.seb;
  const long pr = g.per_rank;
  auto pack = [&](const V6Geom &h, int side, int pa, int pb, int qa, int qb, const double *src) {
    msg[(long)r * pr + h.off + (side ? h.F : 0) + v6_face_index(h, pa, pb, qa, qb)] = *src;
  };
  // the touched points: (jd, n-1) always, (jd+1, 0) with the pair, (0, 0)
  // with the low add
  auto at = [&](int e, int i) { return ur + (long)i * g.spd + (long)e * g.sed; };
  if (d == 2) {
    // points (ix, iy, iz; jx, jy, jz) = (ia, ib, iz; ja, jb, e)
    const int ix = ia, iy = ib;
    const V6Geom &gy = gs.g[1], &gx = gs.g[0];
    const int yside = (iy == 0 && jb == 0) ? 0 : (iy == nz && jb == f.m[1] - 1) ? 1 : -1;
    const int xside = (ix == 0 && ja == 0) ? 0 : (ix == nz && ja == f.m[0] - 1) ? 1 : -1;
    const bool x_interior_y = iy >= 1 && iy <= n - 2;
    if (yside < 0 && (xside < 0 || !x_interior_y)) return;
    auto point = [&](int e, int iz) {
      const double *src = at(e, iz);
      if (yside >= 0) pack(gy, yside, ix, iz, ja, e, src);
      if (xside >= 0 && x_interior_y) pack(gx, xside, iy, iz, jb, e, src);
    };
    point(jd, nz);
    if (jd + 1 < g.md) point(jd + 1, 0);
    if (jd == 0) point(0, 0);
  } else if (d == 1) {
    // points (ix, iy, iz; jx, jy, jz) = (ia, iy, ib; ja, e, jb)
    const int ix = ia, iz = ib;
    const V6Geom &gx = gs.g[0];
    const int xside = (ix == 0 && ja == 0) ? 0 : (ix == nz && ja == f.m[0] - 1) ? 1 : -1;
    if (xside < 0) return;
    auto point = [&](int e, int iy) { pack(gx, xside, iy, iz, e, jb, at(e, iy)); };
    point(jd, nz);
    if (jd + 1 < g.md) point(jd + 1, 0);
    if (jd == 0) point(0, 0);
  }
}

template <typename I>
FACES_HD void v6_part_pack_item(const FieldDesc &f, const V6Geoms &gs, int d, double *msg, int compute, I t)
{
  const I nn = (I)gs.g[d].n * (I)gs.g[d].n, ne = (I)f.m[0] * (I)f.m[1] * (I)f.m[2];
  const I face = t % nn;
  I e = t / nn;
  const I r = e / ne;
  e -= r * ne;
  const int jx = (int)(e % (I)f.m[0]);
  const I e1 = e / (I)f.m[0];
  v6_part_pack_at<0>(f, gs, d, msg, compute, (int)r, jx, (int)(e1 % (I)f.m[1]), (int)(e1 / (I)f.m[1]), (int)face);
}

template <typename I>
FACES_HD void v6_part_item(const FieldDesc &f, const V6Geom &g, const double *msg, int compute, I t)
{
  const I nn = (I)g.n * (I)g.n, ne = (I)f.m[0] * (I)f.m[1] * (I)f.m[2];
  const I face = t % nn;
  I e = t / nn;
  const I r = e / ne;
  e -= r * ne;
  const int jx = (int)(e % (I)f.m[0]);
  const I e1 = e / (I)f.m[0];
  v6_part_at<0>(f, g, msg, compute, (int)r, jx, (int)(e1 % (I)f.m[1]), (int)(e1 / (I)f.m[1]), (int)face);
}

}  // namespace faces
