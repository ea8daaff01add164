// pack_steps.cuh -- the v-26 pack (gpu/v-26-messages/Faces.cc:243-293): the
// 26 boundary messages of every rank, raw values before any sum, in the
// region order of geom.cuh.  Host- and device-callable: pack_kernel runs one
// block of it per CUDA block, the fused message-mode tile kernel runs the
// same blocks in its prologue, and the CPU replay runs them on the host.
#pragma once

#include "geom.cuh"
#include "rows_setup.cuh"

namespace faces {

// Directions in block order: the six faces, then the twelve edges and the
// eight corners (dir = (dx+1) + 3(dy+1) + 9(dz+1)).
FACES_HD int pack_dir(int i)
{
  switch (i) {
    case 0: return 4;
    case 1: return 10;
    case 2: return 12;
    case 3: return 14;
    case 4: return 16;
    case 5: return 22;
    case 6: return 1;
    case 7: return 3;
    case 8: return 5;
    case 9: return 7;
    case 10: return 9;
    case 11: return 11;
    case 12: return 15;
    case 13: return 17;
    case 14: return 19;
    case 15: return 21;
    case 16: return 23;
    case 17: return 25;
    case 18: return 0;
    case 19: return 2;
    case 20: return 6;
    case 21: return 8;
    case 22: return 18;
    case 23: return 20;
    case 24: return 24;
    default: return 26;
  }
}

// The pack's block grid: rows 0 .. nranks*6-1 hold one face message each
// (rank, face), the row's gx blocks striding over it (about two waves of 8
// blocks per SM over all face rows); the rows beyond hold one edge or corner
// message per block (nranks*20 of them).  wide: positions need 64 bits.
struct PackGrid {
  int gx, gy;
  bool wide;
};

inline PackGrid pack_grid(const FieldDesc &f)
{
  const int dface[3][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
  const int dedge[3][3] = {{0, 1, 1}, {1, 0, 1}, {1, 1, 0}};
  long face = 0, edge = 1;
  for (int a = 0; a < 3; a++) {
    face = face > region_size(f, dface[a]) ? face : region_size(f, dface[a]);
    edge = edge > region_size(f, dedge[a]) ? edge : region_size(f, dedge[a]);
  }
  const long face_rows = (long)f.nranks * 6, small = (long)f.nranks * 20;
  long bx = (face + 255) / 256;
  const long want = (152L * 8 * 2 + face_rows - 1) / face_rows;
  if (bx > want) bx = want;
  if (bx < 1) bx = 1;
  PackGrid g;
  g.gx = (int)bx;
  g.gy = (int)(face_rows + (small + bx - 1) / bx);
  g.wide = !(face + 256L * bx < (1L << 31) && edge < (1L << 30));
  return g;
}

struct PackNoTouch {
  FACES_HD void operator()(const double *) const {}
};

// Block (bx, by) of the pack grid (gx blocks per row), thread t of T.  The
// free axes' coordinates come from I-typed divisions (32-bit where the
// message allows), the source offset from per-axis strides set up once per
// block: per point two or three divisions and one load.  touch(p) is called
// with each field address read (the replay records them).
template <typename I, class Touch = PackNoTouch>
FACES_HD void pack_block(const FieldDesc &f, int by, int bx, int gx, int t, int T, Touch touch = Touch())
{
  const int face_rows = f.nranks * 6;
  int r, dir;
  I part, parts;
  if (by < face_rows) {
    r = by / 6;
    dir = pack_dir(by % 6);
    part = (I)bx;
    parts = (I)gx;
  } else {
    const int e = (by - face_rows) * gx + bx;
    if (e >= f.nranks * 20) return;
    r = e / 20;
    dir = pack_dir(6 + e % 20);
    part = 0;
    parts = 1;
  }
  const int rd = r * 27 + dir;
  if (f.msg_off[rd] < 0) return;
  const int d[3] = {dir % 3 - 1, (dir / 3) % 3 - 1, dir / 9 - 1};
  const long n = f.n;
  // fixed axes: the boundary row of the boundary element; free axes in
  // ascending order, the message's i-then-j position order (region_pos).
  // Scalars, not arrays indexed by axis, so that nothing goes to local memory.
  long base = (long)r * f.R, si0 = 0, sj0 = 0, si1 = 0, sj1 = 0;
  int nfree = 0, m0 = 1;
#pragma unroll
  for (int a = 0; a < 3; a++) {
    const long sia = a == 0 ? 1 : a == 1 ? n : n * n;
    const long sja = a == 0 ? n * n * n : a == 1 ? f.sjy : f.sjz;
    if (d[a] == 0) {
      if (nfree == 0) {
        si0 = sia;
        sj0 = sja;
        m0 = f.m[a];
      } else {
        si1 = sia;
        sj1 = sja;
      }
      nfree++;
    } else if (d[a] > 0) {
      base += (n - 1) * sia + (long)(f.m[a] - 1) * sja;
    }
  }
  const I sz = (I)region_size(f, d);
  double *out = f.msg + f.msg_off[rd];
  const double *ur = f.u + base;
  const I nn = (I)(nfree == 2 ? n * n : n), nI = (I)n, mI = (I)m0;
  auto source = [&](I pos) -> long {
    if (nfree == 0) return 0;
    const I q = pos % nn, e = pos / nn;
    if (nfree == 1) return (long)q * si0 + (long)e * sj0;
    return (long)(q % nI) * si0 + (long)(q / nI) * si1 + (long)(e % mI) * sj0 + (long)(e / mI) * sj1;
  };
  // the thread's positions pos, pos + S, pos + 2S, ... (S = parts * T), two
  // at a time with both loads issued before either store, so that their
  // latencies overlap (a store could alias a later load, so the compiler
  // keeps them in order otherwise)
  const I S = parts * (I)T;
  for (I pos = part * (I)T + (I)t; pos < sz; pos += 2 * S) {
    const I pos2 = pos + S;
    const bool two = pos2 < sz;
    const long src = source(pos), src2 = two ? source(pos2) : 0;
    touch(ur + src);
    if (two) touch(ur + src2);
    const double v = ur[src], v2 = two ? ur[src2] : 0.0;
    out[pos] = v;
    if (two) out[pos2] = v2;
  }
}

}  // namespace faces
