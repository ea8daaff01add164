// seam_steps.cuh -- the seam step for direct-mode fields: one thread per
// shared point, no shared memory and no block barrier (host- and
// device-callable, so that tests/native/ptile_emu.cu replays it on the CPU).
//
// The point-per-thread form of the reference's fused inner kernel
// (gpu/v-26-messages/Faces.cc:301-343, one thread per (i0, i1) of an element
// doing its lower z, y and x faces, threads with i1 == 1 its edges), made
// uniform: element e owns the points of its three lower seam planes,
//   plane 0  iz = 0:  (ix, iy) in [0, n-1)^2            (if e has a z-lower neighbour)
//   plane 1  iy = 0:  (ix, iz) in [0, n-1)^2, iz > 0 where plane 0 exists
//   plane 2  ix = 0:  (iy, iz) in [0, n-1)^2, iy > 0 where plane 1 exists,
//                     iz > 0 where plane 0 exists
// so every shared point with all local coordinates below n-1 has one owner.
// A slot's point has 2 copies along each dimension where its coordinate is 0
// and the lower neighbour exists: a face point 2, an edge 4, a corner 8.  The
// thread reads them all, sums them as a tree -- x pairs (lower copy first),
// then y, then z -- and stores the sum in every copy.  Points with a local
// coordinate n-1 that no slot covers lie on an open upper boundary plane of
// the subdomain; gather_point takes them (the planes are 2-D, a small part).
//
// A thread takes one slot (a, b) of an element and the slot's point on each
// plane (like the reference's thread (i0, i1)); a block walks x-chunks of E
// elements of one column (rank, jy, jz), its threads the chunk's slots in
// order, so consecutive threads read consecutive ix (planes 0 and 1) or
// consecutive rows (plane 2).
#pragma once

#include "geom.cuh"
#include "rows_setup.cuh"

namespace faces {

// ---------------------------------------------------------------------------
// gather_point: any point, any mode (also the gather step's body)
// ---------------------------------------------------------------------------

// Rank-local point coordinate g in [0, m*(n-1)] along one axis: element E
// holds g = E*(n-1)+i.  A point with g % (n-1) == 0 has a lower copy (E-1,
// n-1) and an upper copy (E, 0); elements -1 and m belong to the neighbours.
// Scalars (and loops unrolled over fixed bounds below), so that no array is
// indexed at run time and nothing goes to local memory.
struct Copies {
  int cnt, e0, i0, e1, i1;
};

FACES_HD Copies local_axis(int g, int n)
{
  const int nm1 = n - 1, E = g / nm1, i = g % nm1;
  if (i) return Copies{1, E, i, E, i};
  return Copies{2, E - 1, nm1, E, 0};
}

// what the steps below report of each copy they read and write (the CPU
// replay records them; on the device this does nothing)
struct NoTouch {
  FACES_HD void operator()(const double *) const {}
};

// One shared point: point g (global in rank r's subdomain) and its copies,
// summed as a tree x, y, z and written to every local copy.  Points that are
// not shared, or that another rank owns (direct mode), return at once.
template <class Touch = NoTouch>
FACES_HD void gather_point(const FieldDesc &f, int r, const int g[3], int compute, Touch touch = Touch())
{
  const int n = f.n, nm1 = n - 1;
  // a point is shared only if it lies on an element boundary somewhere
  if (g[0] % nm1 && g[1] % nm1 && g[2] % nm1) return;
  bool onb = false, skip = false;
  Copies c[3];
#pragma unroll
  for (int a = 0; a < 3; a++) {
    const int Ga = f.m[a] * nm1;
    onb |= (g[a] == 0 || g[a] == Ga);
    // direct mode: the upper rank owns the points of the shared plane
    if (f.mode == kDirect && g[a] == Ga && nbr_of(f, r, dir_index(a == 0, a == 1, a == 2)) >= 0) skip = true;
    Copies x = local_axis(g[a], n);
    // drop copies whose neighbour rank does not exist
    auto exists = [&](int e) {
      const int dv = e < 0 ? -1 : (e >= f.m[a] ? 1 : 0);
      return dv == 0 || nbr_of(f, r, dir_index(a == 0 ? dv : 0, a == 1 ? dv : 0, a == 2 ? dv : 0)) >= 0;
    };
    const bool ok0 = exists(x.e0), ok1 = x.cnt == 2 && exists(x.e1);
    if (!ok0) { x.e0 = x.e1; x.i0 = x.i1; }
    x.cnt = (int)ok0 + (int)ok1;
    c[a] = x;
  }
  if (skip) return;
  if (c[0].cnt * c[1].cnt * c[2].cnt < 2) return;
  if (!compute && !onb) return;
  double v[2][2][2];
  double *w[2][2][2];
#pragma unroll
  for (int bz = 0; bz < 2; bz++)
#pragma unroll
    for (int by = 0; by < 2; by++)
#pragma unroll
      for (int bx = 0; bx < 2; bx++) {
        w[bz][by][bx] = nullptr;
        v[bz][by][bx] = 0.0;
        if (bz >= c[2].cnt || by >= c[1].cnt || bx >= c[0].cnt) continue;
        const int e[3] = {bx ? c[0].e1 : c[0].e0, by ? c[1].e1 : c[1].e0, bz ? c[2].e1 : c[2].e0};
        const int i[3] = {bx ? c[0].i1 : c[0].i0, by ? c[1].i1 : c[1].i0, bz ? c[2].i1 : c[2].i0};
        int d[3], j[3];
#pragma unroll
        for (int a = 0; a < 3; a++) {
          d[a] = e[a] < 0 ? -1 : (e[a] >= f.m[a] ? 1 : 0);
          j[a] = e[a] < 0 ? f.m[a] - 1 : (e[a] >= f.m[a] ? 0 : e[a]);
        }
        const int dir = dir_index(d[0], d[1], d[2]);
        if (dir == 13 || f.mode == kDirect) {
          const int q = (dir == 13) ? r : nbr_of(f, r, dir);
          double *ptr = f.u + (long)q * f.R + elem_index(f, i[0], i[1], i[2], j[0], j[1], j[2]);
          touch(ptr);
          w[bz][by][bx] = ptr;
          v[bz][by][bx] = *ptr;
        } else {
          const double *rb = recv_of(f, r, dir);
          v[bz][by][bx] = rb[region_pos(f, d, i, j)];
        }
      }
  double sy[2];
#pragma unroll
  for (int bz = 0; bz < 2; bz++) {
    double sx[2];
#pragma unroll
    for (int by = 0; by < 2; by++) sx[by] = (c[0].cnt == 2) ? v[bz][by][0] + v[bz][by][1] : v[bz][by][0];
    sy[bz] = (c[1].cnt == 2) ? sx[0] + sx[1] : sx[0];
  }
  const double s = (c[2].cnt == 2) ? sy[0] + sy[1] : sy[0];
#pragma unroll
  for (int bz = 0; bz < 2; bz++)
#pragma unroll
    for (int by = 0; by < 2; by++)
#pragma unroll
      for (int bx = 0; bx < 2; bx++)
        if (w[bz][by][bx]) *w[bz][by][bx] = s;
}

// ---------------------------------------------------------------------------
// the seam step
// ---------------------------------------------------------------------------

// slots per element: (a, b) in [0, n-1)^2, one point of each plane
FACES_HD constexpr int seam_slots(int n) { return (n - 1) * (n - 1); }

// the base (doubles from f.u) of element (jx, jy, jz) of rank r, where an
// index of -1 is element m-1 of the lower neighbour rank; 0 if that rank does
// not exist (the caller's flags keep such a base unused)
template <int N>
FACES_HD long seam_base(const FieldDesc &f, int r, int jx, int jy, int jz)
{
  const int dx = jx < 0 ? -1 : 0, dy = jy < 0 ? -1 : 0, dz = jz < 0 ? -1 : 0;
  if (dx) jx = f.m[0] - 1;
  if (dy) jy = f.m[1] - 1;
  if (dz) jz = f.m[2] - 1;
  int q = r;
  if (dx | dy | dz) {
#ifdef __CUDA_ARCH__
    q = __ldg(f.nbr + r * 27 + dir_index(dx, dy, dz));
#else
    q = nbr_of(f, r, dir_index(dx, dy, dz));
#endif
  }
  if (q < 0) return 0;
  return (long)q * f.R + (long)jz * f.sjz + (long)jy * f.sjy + (long)jx * (N * N * N);
}

// One x-chunk: nk elements from jx0 of column (r, jy, jz).  b0..b3: element
// jx0 of the column itself, its y-lower, z-lower and y-and-z-lower columns;
// x0..x3: element jx0-1 of the same four columns.  Named members, not an
// array, so that nothing is indexed at run time.
struct SeamChunk {
  long b0, b1, b2, b3, x0, x1, x2, x3;
  int nk;
  bool ylo, zlo, xlo0;  // the y-lower and z-lower columns exist; element jx0-1 exists
};

template <int N>
FACES_HD SeamChunk seam_chunk(const FieldDesc &f, int r, int jy, int jz, int jx0, int nk)
{
  SeamChunk c;
  c.nk = nk;
  c.ylo = jy > 0 || nbr_of(f, r, dir_index(0, -1, 0)) >= 0;
  c.zlo = jz > 0 || nbr_of(f, r, dir_index(0, 0, -1)) >= 0;
  c.xlo0 = jx0 > 0 || nbr_of(f, r, dir_index(-1, 0, 0)) >= 0;
  c.b0 = seam_base<N>(f, r, jx0, jy, jz);
  c.b1 = seam_base<N>(f, r, jx0, jy - 1, jz);
  c.b2 = seam_base<N>(f, r, jx0, jy, jz - 1);
  c.b3 = seam_base<N>(f, r, jx0, jy - 1, jz - 1);
  c.x0 = seam_base<N>(f, r, jx0 - 1, jy, jz);
  c.x1 = seam_base<N>(f, r, jx0 - 1, jy - 1, jz);
  c.x2 = seam_base<N>(f, r, jx0 - 1, jy, jz - 1);
  c.x3 = seam_base<N>(f, r, jx0 - 1, jy - 1, jz - 1);
  return c;
}

// The point of plane `plane` at slot (a, b) of element k of a chunk, any
// number of copies: each copy is read, the copies are summed as a tree (x,
// y, z; lower copy first) and the sum is written to every copy.
template <int N, class Touch>
FACES_HD void seam_point(double *__restrict__ u, const SeamChunk &c, int k, bool xl, int plane, int a, int b,
                         Touch touch)
{
  constexpr long N3 = (long)N * N * N;
  int ix, iy, iz;
  if (plane == 0) {
    if (!c.zlo) return;
    ix = a;
    iy = b;
    iz = 0;
  } else if (plane == 1) {
    if (!c.ylo || (b == 0 && c.zlo)) return;
    ix = a;
    iy = 0;
    iz = b;
  } else {
    if (!xl || (a == 0 && c.ylo) || (b == 0 && c.zlo)) return;
    ix = 0;
    iy = a;
    iz = b;
  }
  const bool cx = ix == 0 && xl, cy = iy == 0 && c.ylo, cz = iz == 0 && c.zlo;
  // element k of each column, and the element before it (x-lower)
  const long ko = (long)k * N3, kl = (long)(k - 1) * N3;
  const long e0 = c.b0 + ko, e1 = c.b1 + ko, e2 = c.b2 + ko, e3 = c.b3 + ko;
  const long l0 = k > 0 ? c.b0 + kl : c.x0, l1 = k > 0 ? c.b1 + kl : c.x1;
  const long l2 = k > 0 ? c.b2 + kl : c.x2, l3 = k > 0 ? c.b3 + kl : c.x3;
  // index 1: the point's own coordinate in that dimension; index 0: the
  // lower copy (coordinate n-1 of the lower element)
  const long px = ix, py = (long)iy * N, pz = (long)iz * N * N;
  constexpr long hx = N - 1, hy = (long)(N - 1) * N, hz = (long)(N - 1) * N * N;
  double *w[2][2][2];
  double v[2][2][2];
#pragma unroll
  for (int bz = 0; bz < 2; bz++)
#pragma unroll
    for (int by = 0; by < 2; by++) {
      // the column: y-lower when by == 0, z-lower when bz == 0
      const long own = bz ? (by ? e0 : e1) : (by ? e2 : e3);
      const long low = bz ? (by ? l0 : l1) : (by ? l2 : l3);
      const long yz = (by ? py : hy) + (bz ? pz : hz);
#pragma unroll
      for (int bx = 0; bx < 2; bx++) {
        const bool live = (bz || cz) && (by || cy) && (bx || cx);
        w[bz][by][bx] = live ? u + (bx ? own + px : low + hx) + yz : nullptr;
        if (live) touch(w[bz][by][bx]);
        v[bz][by][bx] = live ? *w[bz][by][bx] : 0.0;
      }
    }
  double sy[2];
#pragma unroll
  for (int bz = 0; bz < 2; bz++) {
    double sx[2];
#pragma unroll
    for (int by = 0; by < 2; by++) sx[by] = cx ? v[bz][by][0] + v[bz][by][1] : v[bz][by][1];
    sy[bz] = cy ? sx[0] + sx[1] : sx[1];
  }
  const double s = cz ? sy[0] + sy[1] : sy[1];
#pragma unroll
  for (int bz = 0; bz < 2; bz++)
#pragma unroll
    for (int by = 0; by < 2; by++)
#pragma unroll
      for (int bx = 0; bx < 2; bx++)
        if (w[bz][by][bx]) *w[bz][by][bx] = s;
}

// Slot q of a chunk (q < nk * seam_slots(N)): element k = q / slots, then
// (a, b) with a fastest; the slot's point on each plane.  With a, b >= 1 the
// three points are plain face pairs -- z (a, b, 0), y (a, 0, b), x (0, a, b),
// each its own copy plus the lower neighbour's (lower copy first in the sum)
// -- and all six copies are read before any is written; otherwise the points
// lie on edges or a corner and take seam_point.
// a slot whose three points are face pairs (a, b >= 1): the six copies
struct SeamFaces {
  double *z0, *z1, *y0, *y1, *x0, *x1;
  double vz0, vz1, vy0, vy1, vx0, vx1;
  bool xl;
};

template <int N>
FACES_HD bool seam_slot(int q, int &k, int &a, int &b)
{
  constexpr int M = N - 1, P = M * M;
  k = q / P;
  const int p = q - k * P;
  b = p / M;
  a = p - b * M;
  return a > 0 && b > 0;
}

template <int N, class Touch>
FACES_HD void seam_faces_load(double *__restrict__ u, const SeamChunk &c, int k, int a, int b, SeamFaces &s,
                              Touch touch)
{
  constexpr long N3 = (long)N * N * N, NN = (long)N * N;
  s.xl = k > 0 || c.xlo0;
  const long ko = (long)k * N3;
  const long own = c.b0 + ko, xlow = k > 0 ? own - N3 : c.x0;
  s.z1 = u + own + a + (long)b * N;
  s.z0 = u + c.b2 + ko + a + (long)b * N + (N - 1) * NN;
  s.y1 = u + own + a + b * NN;
  s.y0 = u + c.b1 + ko + a + (long)(N - 1) * N + b * NN;
  s.x1 = u + own + (long)a * N + b * NN;
  s.x0 = u + xlow + (N - 1) + (long)a * N + b * NN;
  if (c.zlo) { touch(s.z0); touch(s.z1); }
  if (c.ylo) { touch(s.y0); touch(s.y1); }
  if (s.xl) { touch(s.x0); touch(s.x1); }
  s.vz0 = c.zlo ? *s.z0 : 0.0;
  s.vz1 = c.zlo ? *s.z1 : 0.0;
  s.vy0 = c.ylo ? *s.y0 : 0.0;
  s.vy1 = c.ylo ? *s.y1 : 0.0;
  s.vx0 = s.xl ? *s.x0 : 0.0;
  s.vx1 = s.xl ? *s.x1 : 0.0;
}

FACES_HD void seam_faces_store(const SeamChunk &c, const SeamFaces &s)
{
  if (c.zlo) {
    const double v = s.vz0 + s.vz1;
    *s.z0 = v;
    *s.z1 = v;
  }
  if (c.ylo) {
    const double v = s.vy0 + s.vy1;
    *s.y0 = v;
    *s.y1 = v;
  }
  if (s.xl) {
    const double v = s.vx0 + s.vx1;
    *s.x0 = v;
    *s.x1 = v;
  }
}

// the points of a slot with a == 0 or b == 0 (edges, the corner)
template <int N, class Touch>
FACES_HD void seam_edges(double *__restrict__ u, const SeamChunk &c, int k, int a, int b, Touch touch)
{
  const bool xl = k > 0 || c.xlo0;
  seam_point<N>(u, c, k, xl, 0, a, b, touch);
  seam_point<N>(u, c, k, xl, 1, a, b, touch);
  seam_point<N>(u, c, k, xl, 2, a, b, touch);
}

template <int N, class Touch = NoTouch>
FACES_HD void seam_item(double *__restrict__ u, const SeamChunk &c, int q, Touch touch = Touch())
{
  int k, a, b;
  if (!seam_slot<N>(q, k, a, b)) {
    seam_edges<N>(u, c, k, a, b, touch);
    return;
  }
  SeamFaces s;
  seam_faces_load<N>(u, c, k, a, b, s, touch);
  seam_faces_store(c, s);
}

// the work item w (a chunk) -> rank, column and first element
struct SeamUnit {
  int r, jy, jz, jx0, nk;
};

FACES_HD SeamUnit seam_unit(const FieldDesc &f, int E, int nch, long w)
{
  SeamUnit s;
  const int c = (int)(w % nch);
  long rest = w / nch;
  s.jy = (int)(rest % f.m[1]);
  rest /= f.m[1];
  s.jz = (int)(rest % f.m[2]);
  s.r = (int)(rest / f.m[2]);
  s.jx0 = c * E;
  s.nk = f.m[0] - s.jx0 < E ? f.m[0] - s.jx0 : E;
  return s;
}

// The open upper boundary planes: g_d = m_d*(n-1) where rank r has no upper
// neighbour along d; the x plane, the y plane without the x plane's points,
// the z plane without both.  Only a plane's seam lines hold shared points
// (a coordinate g_a or g_b that is a multiple of n-1, a < b the other two
// dimensions): per plane the lines along b at the seams of a, then the lines
// along a at the seams of b without the points already taken.  Each rank has
// a fixed range of items (the three planes' counts without the exclusions);
// items of planes that are not open, or past a plane's count, do nothing.
FACES_HD long seam_plane_capacity(const FieldDesc &f, int d)
{
  const int a = d == 0 ? 1 : 0, b = d == 2 ? 1 : 2;
  const long nm1 = f.n - 1, Ga = f.m[a] * nm1 + 1, Gb = f.m[b] * nm1 + 1;
  return (f.m[a] + 1) * Gb + (f.m[b] + 1) * (Ga - f.m[a] - 1);
}

FACES_HD long seam_plane_items(const FieldDesc &f)
{
  return seam_plane_capacity(f, 0) + seam_plane_capacity(f, 1) + seam_plane_capacity(f, 2);
}

template <class Touch = NoTouch>
FACES_HD void seam_plane_point(const FieldDesc &f, long p, Touch touch = Touch())
{
  const long per = seam_plane_items(f);
  const int r = (int)(p / per);
  long t = p - (long)r * per;
  const int nm1 = f.n - 1;
  const bool ox = nbr_of(f, r, dir_index(1, 0, 0)) < 0, oy = nbr_of(f, r, dir_index(0, 1, 0)) < 0;
  const bool oz = nbr_of(f, r, dir_index(0, 0, 1)) < 0;
  int d = 0;
  while (d < 2 && t >= seam_plane_capacity(f, d)) t -= seam_plane_capacity(f, d++);
  if (!(d == 0 ? ox : d == 1 ? oy : oz)) return;
  const int a = d == 0 ? 1 : 0, b = d == 2 ? 1 : 2;
  // the plane's extent along a and b: an earlier open plane's points excluded
  // (a is x in the y and z planes, b is y in the z plane)
  const long Wa = f.m[a] * (long)nm1 + 1 - (d > 0 && ox ? 1 : 0);
  const long Wb = f.m[b] * (long)nm1 + 1 - (d == 2 && oy ? 1 : 0);
  const long Sa = (Wa - 1) / nm1 + 1, Sb = (Wb - 1) / nm1 + 1;  // seam coordinates in range
  long ga, gb;
  if (t < Sa * Wb) {
    ga = (t / Wb) * nm1;
    gb = t % Wb;
  } else {
    t -= Sa * Wb;
    const long rest = Wa - Sa;  // coordinates along a off the seams
    if (rest <= 0 || t >= Sb * rest) return;
    gb = (t / rest) * nm1;
    const long i = t % rest;
    ga = (i / (nm1 - 1)) * nm1 + i % (nm1 - 1) + 1;
  }
  int g[3];
  g[d] = f.m[d] * nm1;
  g[a] = (int)ga;
  g[b] = (int)gb;
  gather_point(f, r, g, 1, touch);
}

// ---------------------------------------------------------------------------
// The lean form (the thread layout of the reference's fused inner kernel,
// gpu/v-26-messages/Faces.cc:301-343): one thread per face slot (a, b) in
// [1, n-2]^2 of every element, which does the slot's three face pairs one
// after the other; the threads with b == 1 also do the three edge points at
// coordinate a -- (a, 0, 0), (0, a, 0), (0, 0, a) -- and the thread (1, 1)
// the corner, while the element's sectors are still in cache.  Few
// registers and no per-chunk state, so that many warps are resident.  The
// open boundary planes take a second launch (non-periodic fields only).  A
// face point has one zero coordinate, an edge point two, the corner three, a
// boundary-plane point a coordinate n-1: the sets are disjoint.  For n = 2
// an element has no face or edge points: its one thread does the corner.
// ---------------------------------------------------------------------------

FACES_HD constexpr int seam_lean_slots(int n) { return n > 2 ? (n - 2) * (n - 2) : 1; }

// an element of the field
struct SeamElem {
  int r, jx, jy, jz;
};

// The element (jx+dx, jy+dy, jz+dz) of rank r, dx, dy, dz in {-1, 0}, and
// whether it exists (a lower index of -1 is the lower neighbour rank's last
// element)
template <int N>
FACES_HD bool seam_elem_at(const FieldDesc &f, const SeamElem &el, int dx, int dy, int dz, long &base)
{
  const bool wx = dx && el.jx == 0, wy = dy && el.jy == 0, wz = dz && el.jz == 0;
  int q = el.r;
  if (wx || wy || wz) {
#ifdef __CUDA_ARCH__
    q = __ldg(f.nbr + el.r * 27 + dir_index(wx ? -1 : 0, wy ? -1 : 0, wz ? -1 : 0));
#else
    q = nbr_of(f, el.r, dir_index(wx ? -1 : 0, wy ? -1 : 0, wz ? -1 : 0));
#endif
    if (q < 0) return false;
  }
  const int jx = wx ? f.m[0] - 1 : el.jx + dx, jy = wy ? f.m[1] - 1 : el.jy + dy;
  const int jz = wz ? f.m[2] - 1 : el.jz + dz;
  base = (long)q * f.R + (long)jz * f.sjz + (long)jy * f.sjy + (long)jx * (N * N * N);
  return true;
}

// Edge point at coordinate a of the line along `line` (0: (a, 0, 0), 1:
// (0, a, 0), 2: (0, 0, a)): a copy for each lower neighbour along its two
// zero dimensions p < q that exists (2 or 4 copies; 1: nothing to do),
// summed p first (x before y before z), lower copy first.
template <int N, class Touch>
FACES_HD void seam_edge_point(const FieldDesc &f, const SeamElem &el, long own, int line, int a, Touch touch)
{
  constexpr long NN = (long)N * N;
  const int p = line == 0 ? 1 : 0, q = line == 2 ? 1 : 2;
  const long along = line == 0 ? a : line == 1 ? (long)a * N : (long)a * NN;
  const long hp = p == 0 ? N - 1 : (long)(N - 1) * N, hq = q == 1 ? (long)(N - 1) * N : (long)(N - 1) * NN;
  long b10 = 0, b01 = 0, b00 = 0;  // [q side][p side], 1 = this element's side
  const bool lp = seam_elem_at<N>(f, el, p == 0 ? -1 : 0, p == 1 ? -1 : 0, 0, b10);
  const bool lq = seam_elem_at<N>(f, el, 0, q == 1 ? -1 : 0, q == 2 ? -1 : 0, b01);
  if (!lp && !lq) return;
  const bool lpq = lp && lq && seam_elem_at<N>(f, el, p == 0 ? -1 : 0, p == 1 || q == 1 ? -1 : 0, q == 2 ? -1 : 0, b00);
  double *c11 = f.u + own + along, *c10 = f.u + b10 + along + hp;
  double *c01 = f.u + b01 + along + hq, *c00 = f.u + b00 + along + hp + hq;
  touch(c11);
  if (lp) touch(c10);
  if (lq) touch(c01);
  if (lpq) touch(c00);
  const double v11 = *c11, v10 = lp ? *c10 : 0.0, v01 = lq ? *c01 : 0.0, v00 = lpq ? *c00 : 0.0;
  const double sq0 = lp ? v00 + v01 : v01;
  const double sq1 = lp ? v10 + v11 : v11;
  const double t = lq ? sq0 + sq1 : sq1;
  *c11 = t;
  if (lp) *c10 = t;
  if (lq) *c01 = t;
  if (lpq) *c00 = t;
}

// the corner (0, 0, 0): up to 8 copies, one tree over x, y, z.  The copies
// are visited in tree order with one running sum per level (the first copy
// of a level starts it, the next is added), and their addresses are found
// again for the stores: one thread per element takes it, so it keeps few
// registers rather than many loads in flight.
template <int N, class Touch>
FACES_HD void seam_corner(const FieldDesc &f, const SeamElem &el, Touch touch)
{
  constexpr long NN = (long)N * N;
  long base = 0;
  const bool cx = seam_elem_at<N>(f, el, -1, 0, 0, base), cy = seam_elem_at<N>(f, el, 0, -1, 0, base);
  const bool cz = seam_elem_at<N>(f, el, 0, 0, -1, base);
  if (!cx && !cy && !cz) return;
  const int x0 = cx ? 0 : 1, y0 = cy ? 0 : 1, z0 = cz ? 0 : 1;
  auto at = [&](int bx, int by, int bz) {
    long i = 0;
    seam_elem_at<N>(f, el, bx - 1, by - 1, bz - 1, i);
    return i + (bx ? 0 : N - 1) + (by ? 0 : (N - 1) * N) + (bz ? 0 : (N - 1) * NN);
  };
  double tz = 0.0;
#pragma unroll 1
  for (int bz = z0; bz < 2; bz++) {
    double ty = 0.0;
#pragma unroll 1
    for (int by = y0; by < 2; by++) {
      double tx = 0.0;
#pragma unroll 1
      for (int bx = x0; bx < 2; bx++) {
        const long i = at(bx, by, bz);
        touch(f.u + i);
        const double v = f.u[i];
        tx = bx == x0 ? v : tx + v;
      }
      ty = by == y0 ? tx : ty + tx;
    }
    tz = bz == z0 ? ty : tz + ty;
  }
#pragma unroll 1
  for (int k = 0; k < 8; k++) {
    const int bx = k & 1, by = (k >> 1) & 1, bz = k >> 2;
    if (bx >= x0 && by >= y0 && bz >= z0) f.u[at(bx, by, bz)] = tz;
  }
}

// The three face pairs of face slot (a, b) of element el (a, b in [1, n-2]):
// this element's copies (a, b, 0), (a, 0, b), (0, a, b) and the z-, y- and
// x-lower elements' copies at n-1 along the pair's axis; each sum lower copy
// first.  The six points are distinct, so every load is issued before any
// store: their memory latencies overlap instead of following one another.
template <int N, class Touch>
FACES_HD void seam_face_pairs(const FieldDesc &f, const SeamElem &el, long own, int a, int b, Touch touch)
{
  constexpr long NN = (long)N * N;
  long lz = 0, ly = 0, lx = 0;
  const bool hz = seam_elem_at<N>(f, el, 0, 0, -1, lz);
  const bool hy = seam_elem_at<N>(f, el, 0, -1, 0, ly);
  const bool hx = seam_elem_at<N>(f, el, -1, 0, 0, lx);
  const long oz = a + (long)b * N, oy = a + (long)b * NN, ox = (long)a * N + (long)b * NN;
  double *z1 = f.u + own + oz, *z0 = f.u + lz + oz + (N - 1) * NN;
  double *y1 = f.u + own + oy, *y0 = f.u + ly + oy + (long)(N - 1) * N;
  double *x1 = f.u + own + ox, *x0 = f.u + lx + ox + (N - 1);
  if (hz) {
    touch(z0);
    touch(z1);
  }
  if (hy) {
    touch(y0);
    touch(y1);
  }
  if (hx) {
    touch(x0);
    touch(x1);
  }
  const double vz0 = hz ? *z0 : 0.0, vz1 = hz ? *z1 : 0.0;
  const double vy0 = hy ? *y0 : 0.0, vy1 = hy ? *y1 : 0.0;
  const double vx0 = hx ? *x0 : 0.0, vx1 = hx ? *x1 : 0.0;
  if (hz) {
    const double v = vz0 + vz1;
    *z0 = v;
    *z1 = v;
  }
  if (hy) {
    const double v = vy0 + vy1;
    *y0 = v;
    *y1 = v;
  }
  if (hx) {
    const double v = vx0 + vx1;
    *x0 = v;
    *x1 = v;
  }
}

// lean item t of column col (rank, jz, jy; jy fastest): element t /
// seam_lean_slots(n) of the column, slot (a, b) in [1, n-2]^2 with a fastest
// (32-bit decoding: a column holds at most 2^31 items)
template <int N, class Touch = NoTouch>
FACES_HD void seam_lean_item(const FieldDesc &f, int col, int t, Touch touch = Touch())
{
  constexpr int W = N - 2, F = seam_lean_slots(N);
  constexpr long NN = (long)N * N;
  SeamElem el;
  el.jy = col % f.m[1];
  const int rest = col / f.m[1];
  el.jz = rest % f.m[2];
  el.r = rest / f.m[2];
  el.jx = t / F;
  const int s = t - el.jx * F;
  const long own = (long)el.r * f.R + (long)el.jz * f.sjz + (long)el.jy * f.sjy + (long)el.jx * (N * NN);
  if constexpr (W <= 0) {
    (void)s;
    (void)own;
    seam_corner<N>(f, el, touch);
  } else {
    const int bq = s / W;
    const int a = 1 + s - bq * W, b = 1 + bq;
    seam_face_pairs<N>(f, el, own, a, b, touch);
    if (b == 1) {
      seam_edge_point<N>(f, el, own, 0, a, touch);
      seam_edge_point<N>(f, el, own, 1, a, touch);
      seam_edge_point<N>(f, el, own, 2, a, touch);
      if (a == 1) seam_corner<N>(f, el, touch);
    }
  }
}

}  // namespace faces
