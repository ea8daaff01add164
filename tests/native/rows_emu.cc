// rows_emu.cc -- CPU replay of the row kernel (test infrastructure).
//
// Runs the kernel's own tile/slot setup (faces_gb300/csrc/rows_setup.cuh) for
// every tile and slot of a share and emulates one thread block in lockstep:
// x pairs per slot, then y pairs, then z pairs, then the stores.  Checks that
// every pointer stays inside the field or the message buffers and that no
// field point is written more than once per share.  The message mode's pack
// is replayed from region(d) as the pack kernel does.
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "geom.cuh"
#include "rows_setup.cuh"
#include "tables.h"
#include "tile_ops.cuh"

using namespace faces;

namespace {

struct Ctx {
  FieldDesc f;
  const double *u0, *u1, *m0, *m1;
  std::vector<unsigned char> wcount;
  std::string err;
  bool ok = true;
  long regular_tiles = 0, all_tiles = 0;
};

bool in_field(const Ctx &c, const double *p, long len)
{
  return p >= c.u0 && p + len <= c.u1;
}

bool in_any(const Ctx &c, const double *p, long len)
{
  return in_field(c, p, len) || (c.m0 && p >= c.m0 && p + len <= c.m1);
}

void bad(Ctx &c, const char *what, long tile, int sy, int sz, int jx)
{
  if (!c.ok) return;
  char buf[256];
  snprintf(buf, sizeof(buf), "%s (tile %ld slot %d,%d jx %d)", what, tile, sy, sz, jx);
  c.err = buf;
  c.ok = false;
}

void write(Ctx &c, double *p, double v, long tile, int sy, int sz, int jx)
{
  if (!in_field(c, p, 1)) { bad(c, "write outside the field", tile, sy, sz, jx); return; }
  const long k = p - c.u0;
  if (c.wcount[k]++) { bad(c, "point written twice", tile, sy, sz, jx); return; }
  *p = v;
}

void pack(FieldDesc &f)
{
  const int n = f.n;
  for (int r = 0; r < f.nranks; r++)
    for (int dir = 0; dir < 27; dir++) {
      if (dir == 13 || f.msg_off[r * 27 + dir] < 0) continue;
      const int d[3] = {dir % 3 - 1, (dir / 3) % 3 - 1, dir / 9 - 1};
      const long sz = region_size(f, d);
      for (long pos = 0; pos < sz; pos++) {
        int i[3], j[3];
        long t = pos;
        for (int a = 0; a < 3; a++)
          if (d[a] == 0) { i[a] = (int)(t % n); t /= n; }
        for (int a = 0; a < 3; a++)
          if (d[a] == 0) { j[a] = (int)(t % f.m[a]); t /= f.m[a]; }
        for (int a = 0; a < 3; a++)
          if (d[a] != 0) { i[a] = d[a] < 0 ? 0 : n - 1; j[a] = d[a] < 0 ? 0 : f.m[a] - 1; }
        f.msg[f.msg_off[r * 27 + dir] + pos] = f.u[(long)r * f.R + elem_index(f, i[0], i[1], i[2], j[0], j[1], j[2])];
      }
    }
}

// one tile, all slots in lockstep
void run_tile(Ctx &c, const RowPlan &p, long tile)
{
  const FieldDesc &f = c.f;
  const int n = f.n, P = pow2_at_least(n), NV = n - 1;
  const TileCoords t = tile_coords(f, p, tile);
  if (t.skip) return;
  const int S = P * n;
  std::vector<SlotSetup> ss(S);
  for (int sl = 0; sl < S; sl++) slot_setup(f, t, sl % P, sl / P, P, ss[sl]);
  std::vector<double> carry(S, 0.0), cur(S * n), w(S * NV), wy(S * NV);
  std::vector<char> hc(S, 0);
  std::vector<double *> carry_w(S, nullptr);
  for (int sl = 0; sl < S; sl++) {
    const SlotSetup &s = ss[sl];
    if (s.lo) {
      if (!in_any(c, s.lo, 1)) bad(c, "lo end outside buffers", tile, sl % P, sl / P, -1);
      if (s.lo_w && !in_field(c, s.lo, 1)) bad(c, "writable lo end outside field", tile, sl % P, sl / P, -1);
      if (!c.ok) return;
      carry[sl] = *s.lo;
      hc[sl] = 1;
      carry_w[sl] = s.lo_w ? const_cast<double *>(s.lo) : nullptr;
    }
  }
  auto pairs = [&](int C) {
    // y pairs
    for (int sl = 0; sl < S; sl++) {
      const SlotSetup &s = ss[sl];
      const int sy = sl % P, sz = sl / P;
      for (int k = 0; k < C; k++) wy[sl * NV + k] = w[sl * NV + k];
      if (!s.yseam) continue;
      const int syp = sy == 0 ? n - 1 : 0;
      const int pl = syp + P * sz;
      for (int k = 0; k < C; k++) {
        const double o = w[pl * NV + k];
        wy[sl * NV + k] = s.valid ? (s.pvy ? w[sl * NV + k] + o : w[sl * NV + k]) : o;
      }
    }
    // z pairs
    for (int sl = 0; sl < S; sl++) {
      const SlotSetup &s = ss[sl];
      const int sy = sl % P, sz = sl / P;
      for (int k = 0; k < C; k++) w[sl * NV + k] = wy[sl * NV + k];
      if (!s.zseam) continue;
      const int szp = sz == 0 ? n - 1 : 0;
      const int pl = sy + P * szp;
      const bool ypres = s.valid || s.pvy, pzpres = s.pvz || s.pvyz;
      for (int k = 0; k < C; k++) {
        const double o = wy[pl * NV + k];
        w[sl * NV + k] = ypres ? (pzpres ? wy[sl * NV + k] + o : wy[sl * NV + k]) : o;
      }
    }
  };
  for (int jx = t.jx0; jx < t.jx1; jx++) {
    for (int sl = 0; sl < S; sl++) {
      const SlotSetup &s = ss[sl];
      if (!s.valid) continue;
      const double *row = s.rd + (long)jx * s.es;
      if (!in_any(c, row, n)) { bad(c, "row read outside buffers", tile, sl % P, sl / P, jx); return; }
      for (int k = 0; k < n; k++) cur[sl * n + k] = row[k];
      w[sl * NV] = hc[sl] ? carry[sl] + cur[sl * n] : cur[sl * n];
      for (int k = 1; k < NV; k++) w[sl * NV + k] = cur[sl * n + k];
    }
    pairs(NV);
    for (int sl = 0; sl < S; sl++) {
      const SlotSetup &s = ss[sl];
      if (s.writable) {
        double *row = const_cast<double *>(s.rd) + (long)jx * s.es;
        const bool interior = !(s.yseam || s.zseam);
        if (interior) write(c, row, w[sl * NV], tile, sl % P, sl / P, jx);
        else for (int k = 0; k < NV; k++) write(c, row + k, w[sl * NV + k], tile, sl % P, sl / P, jx);
      }
      if (carry_w[sl]) write(c, carry_w[sl], w[sl * NV], tile, sl % P, sl / P, jx);
      if (!c.ok) return;
      if (s.valid) {
        carry[sl] = cur[sl * n + n - 1];
        hc[sl] = 1;
        carry_w[sl] = s.writable ? const_cast<double *>(s.rd) + (long)jx * s.es + n - 1 : nullptr;
      }
    }
  }
  if (t.hi_x) {
    for (int sl = 0; sl < S; sl++) {
      const SlotSetup &s = ss[sl];
      if (s.hi && !in_any(c, s.hi, 1)) { bad(c, "hi end outside buffers", tile, sl % P, sl / P, f.m[0]); return; }
      w[sl * NV] = s.hi ? carry[sl] + *s.hi : carry[sl];
    }
    pairs(1);
    for (int sl = 0; sl < S; sl++)
      if (carry_w[sl]) write(c, carry_w[sl], w[sl * NV], tile, sl % P, sl / P, f.m[0]);
  }
}

// one tile of the shared-memory tile kernel: copy in, groups, copy out -- the
// same functions the kernel's threads call, run one unit at a time
// concurrency model: every tile of a launch reads the field as it was at the
// launch (snapshot), and inside a tile every group / pass item reads the
// staged cells as they were before the phase -- a read of a cell that
// another tile or item writes then changes the result
const double *g_snap = nullptr;  // field snapshot (same layout as c.u0)

static const double *snap_of(const Ctx &c, const double *g)
{
  if (g_snap && g >= c.u0 && g < c.u1) return g_snap + (g - c.u0);
  return g;
}

// run one phase item by item against a snapshot of the stage: each item
// reads the pre-phase cells and its writes are applied afterwards
template <class F>
static bool phase_concurrent(std::vector<double> &sm, long items, F item, std::string &err)
{
  const std::vector<double> before(sm);
  std::vector<double> out(sm);
  std::vector<unsigned char> owner(sm.size(), 0);
  for (long i = 0; i < items; i++) {
    std::vector<double> work(before);
    item(work.data(), i);
    for (size_t j = 0; j < sm.size(); j++)
      if (std::memcmp(&work[j], &before[j], sizeof(double)) != 0) {
        if (owner[j]++) { err = "staged cell written by two items"; return false; }
        out[j] = work[j];
      }
  }
  sm = out;
  return true;
}

void run_tile_smem(Ctx &c, const RowPlan &p, long tile, int K, std::vector<RowMeta> &prev, long &prev_tile)
{
  const FieldDesc &f = c.f;
  const int n = f.n, NN = n * n;
  const TileCoords t = tile_coords(f, p, tile);
  if (t.skip) return;
  const int nk = t.jx1 - t.jx0;
  const bool hi_x = t.hi_x;
  std::vector<RowMeta> meta(NN);
  for (int r = 0; r < NN; r++) row_meta(f, t, r, meta[r]);
  // the tile kernel's per-slot column state and x ends must reproduce the
  // full setup of every row
  for (int r = 0; r < NN; r++) {
    const SlotCol sc = slot_col(f, t, r);
    const double *lo, *hi;
    const unsigned fl = row_ends(f, t, sc, r, lo, hi);
    if (sc.rd != meta[r].rd || sc.es != meta[r].es || fl != meta[r].flags || lo != meta[r].lo || hi != meta[r].hi) {
      bad(c, "slot column state differs from the full row setup", tile, r % n, r / n, 0);
      return;
    }
  }
  // the kernel reuses the previous chunk's metadata: it must equal the fresh one
  if (prev_tile == tile - 1 && t.c > 0) {
    for (int r = 0; r < NN; r++) {
      RowMeta m;
      tile_row_meta(f, t, true, prev.data(), r, m);
      if (m.rd != meta[r].rd || m.lo != meta[r].lo || m.hi != meta[r].hi || m.es != meta[r].es ||
          m.flags != meta[r].flags) {
        bad(c, "reused row metadata differs from the fresh one", tile, r % n, r / n, 0);
        return;
      }
    }
  }
  prev = meta;
  prev_tile = tile;
  const long stage = tile_stage_doubles(n, K);
  std::vector<double> sm(stage, -12345.0);
  double *buf = sm.data(), *locol = buf + (long)K * NN * smem_row_stride(n), *hicol = locol + NN;
  auto in_smem = [&](const double *q, int len) { return q >= sm.data() && q + len <= sm.data() + stage; };
  const int NP = pieces_per_row(n), PW = piece_doubles(n), RS = smem_row_stride(n);
  // copy in: the end columns, then every slot (r, p) for every element
  for (int r = 0; r < NN; r++) {
    const RowMeta &m = meta[r];
    if (m.flags & kLoOk) {
      if (!in_any(c, m.lo, 1)) { bad(c, "lo end outside buffers", tile, r, 0, 0); return; }
      locol[r] = *snap_of(c, m.lo);
    }
    if (m.flags & kHiOk) {
      if (!in_any(c, m.hi, 1)) { bad(c, "hi end outside buffers", tile, r, 0, 0); return; }
      hicol[r] = *snap_of(c, m.hi);
    }
  }
  for (int sl = 0; sl < NN * NP; sl++) {
    const int r = sl / NP, pc = sl % NP;
    const RowMeta &m = meta[r];
    if (!(m.flags & kRowValid) || !piece_needed(n, m.flags, pc)) continue;
    for (int k = 0; k < nk; k++) {
      Move mv;
      slot_move(n, m, r, pc, t.jx0, k, buf, mv);
      if (!in_any(c, mv.g, mv.len)) { bad(c, "tile copy-in outside buffers", tile, r, pc, k); return; }
      if (!in_smem(mv.s, mv.len) || mv.s + mv.len > locol) { bad(c, "tile copy-in outside its stage", tile, r, pc, k); return; }
      if (mv.len == 2 && (((uintptr_t)mv.g) & 15)) { bad(c, "16-byte copy-in misaligned", tile, r, pc, k); return; }
      if (mv.len == 2 && (((char *)mv.s - (char *)sm.data()) & 15)) { bad(c, "16-byte smem slot misaligned", tile, r, pc, k); return; }
      for (int q = 0; q < mv.len; q++) mv.s[q] = snap_of(c, mv.g)[q];
    }
  }
  bool regular = true;
  for (int r = 0; r < NN; r++) regular = regular && row_regular(meta[r].flags, hi_x);
  c.regular_tiles += regular;
  c.all_tiles++;
  std::string perr;
  const long off_buf = buf - sm.data(), off_lo = locol - sm.data(), off_hi = hicol - sm.data();
  std::vector<unsigned> rflags(NN);
  for (int r = 0; r < NN; r++) rflags[r] = meta[r].flags;
  if (regular) {
    // three dense passes, each item against the pre-pass cells
    for (int pass = 0; pass < 3 && c.ok; pass++) {
      const long items = pass == 0 ? xpass_items(n, nk, hi_x) : yzpass_items(n, nk, hi_x);
      const bool ok = phase_concurrent(sm, items, [&](double *w, long i) {
        if (pass == 0) xpass_item(n, nk, w + off_buf, w + off_lo, w + off_hi, (int)i);
        else yzpass_item(n, nk, hi_x, pass, w + off_buf, w + off_lo, w + off_hi, (int)i);
      }, perr);
      if (!ok) { bad(c, perr.c_str(), tile, pass, 0, 0); return; }
    }
  } else {
    const bool ok = phase_concurrent(sm, tile_groups(n, nk, hi_x), [&](double *w, long g) {
      tile_group(n, nk, rflags.data(), w + off_buf, w + off_lo, w + off_hi, g);
    }, perr);
    if (!ok) { bad(c, perr.c_str(), tile, 0, 0, 0); return; }
  }
  // copy out
  for (int r = 0; r < NN; r++)
    if (meta[r].flags & kLoWritable) write(c, const_cast<double *>(meta[r].lo), locol[r], tile, r, 0, -1);
  for (int sl = 0; sl < NN * NP; sl++) {
    const int r = sl / NP, pc = sl % NP;
    const RowMeta &m = meta[r];
    if (!(m.flags & kRowWritable) || !piece_needed(n, m.flags, pc)) continue;
    for (int k = 0; k < nk; k++) {
      Move mv;
      slot_move(n, m, r, pc, t.jx0, k, buf, mv);
      const int len = slot_out_len(n, nk, hi_x, pc, k);
      for (int q = 0; q < len; q++) write(c, const_cast<double *>(mv.g) + q, mv.s[q], tile, r, pc, k);
      if (!c.ok) return;
    }
  }
  (void)PW; (void)RS;
}

}  // namespace

extern "C" int tiles_emulate(int lx, int ly, int lz, int mx, int my, int mz, int n, int periodic, int messages,
                             int K, double *u, int nsteps, char *err, int errlen, long *regular)
{
  Ctx c;
  FieldDesc &f = c.f;
  f.n = n;
  f.m[0] = mx; f.m[1] = my; f.m[2] = mz;
  f.L[0] = lx; f.L[1] = ly; f.L[2] = lz;
  f.periodic = periodic;
  f.mode = messages ? kMessages : kDirect;
  f.nranks = lx * ly * lz;
  f.sjy = (long)n * n * n * mx;
  f.sjz = jz_stride(n, mx, my);
  f.R = f.sjz * mz;
  f.u = u;
  std::vector<int> nbr = neighbour_table(f.L, periodic != 0);
  std::vector<long> off;
  long mtot = messages ? message_offsets(f, nbr, off) : 0;
  if (!messages) off.assign(nbr.size(), -1);
  std::vector<double> msg(mtot > 0 ? mtot : 1, 0.0);
  std::vector<long> roff = receive_offsets(nbr, off);
  f.nbr = nbr.data();
  f.msg_off = off.data();
  f.recv_off = roff.data();
  f.msg = messages ? msg.data() : nullptr;
  c.u0 = u;
  c.u1 = u + f.R * f.nranks;
  c.m0 = messages ? msg.data() : nullptr;
  c.m1 = messages ? msg.data() + mtot : nullptr;
  const RowPlan p = make_row_plan(f, K, 0);
  std::vector<RowMeta> prev;
  long prev_tile = -2;
  std::vector<double> snap;
  for (int step = 0; step < nsteps && c.ok; step++) {
    c.wcount.assign(f.R * f.nranks, 0);
    if (messages) pack(f);
    snap.assign(u, u + f.R * f.nranks);
    g_snap = snap.data();
    // tiles in reverse order too: any order must give the same field
    for (long tile = 0; tile < p.ntiles && c.ok; tile++)
      run_tile_smem(c, p, (step % 2) ? p.ntiles - 1 - tile : tile, tile_instance_k(p.chunk), prev, prev_tile);
  }
  g_snap = nullptr;
  if (regular) { regular[0] = c.regular_tiles; regular[1] = c.all_tiles; }
  if (!c.ok) {
    snprintf(err, errlen, "%s", c.err.c_str());
    return -1;
  }
  return 0;
}

extern "C" int rows_emulate(int lx, int ly, int lz, int mx, int my, int mz, int n, int periodic, int messages,
                            int chunk, int tiles_per_block, double *u, int nsteps, char *err, int errlen)
{
  Ctx c;
  FieldDesc &f = c.f;
  f.n = n;
  f.m[0] = mx; f.m[1] = my; f.m[2] = mz;
  f.L[0] = lx; f.L[1] = ly; f.L[2] = lz;
  f.periodic = periodic;
  f.mode = messages ? kMessages : kDirect;
  f.nranks = lx * ly * lz;
  f.sjy = (long)n * n * n * mx;
  f.sjz = jz_stride(n, mx, my);
  f.R = f.sjz * mz;
  f.u = u;
  std::vector<int> nbr = neighbour_table(f.L, periodic != 0);
  std::vector<long> off;
  long mtot = messages ? message_offsets(f, nbr, off) : 0;
  if (!messages) off.assign(nbr.size(), -1);
  std::vector<double> msg(mtot > 0 ? mtot : 1, 0.0);
  std::vector<long> roff = receive_offsets(nbr, off);
  f.nbr = nbr.data();
  f.msg_off = off.data();
  f.recv_off = roff.data();
  f.msg = messages ? msg.data() : nullptr;
  c.u0 = u;
  c.u1 = u + f.R * f.nranks;
  c.m0 = messages ? msg.data() : nullptr;
  c.m1 = messages ? msg.data() + mtot : nullptr;
  const RowPlan p = make_row_plan(f, chunk > 0 ? chunk : mx, tiles_per_block);
  for (int step = 0; step < nsteps && c.ok; step++) {
    c.wcount.assign(f.R * f.nranks, 0);
    if (messages) pack(f);
    for (long tile = 0; tile < p.ntiles && c.ok; tile++) run_tile(c, p, tile);
  }
  if (!c.ok) {
    snprintf(err, errlen, "%s", c.err.c_str());
    return -1;
  }
  return 0;
}
