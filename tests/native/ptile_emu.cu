// ptile_emu.cu -- CPU replay of the periodic tile step (test infrastructure).
//
// Compiled by nvcc as host code only: the step's own functions from
// faces_gb300/csrc/ptile_steps.cuh (pstage, pxpass, pyzpass; __host__
// __device__, with cp.async replaced by an immediate copy on the host) run
// for every tile of a share, thread by thread, for a team of T threads (256:
// the block form, 32: the warp form) and any tile length K -- the single-
// field kernel's powers of 2 and the batched kernel's stage-filling lengths.
//
// Concurrency model:
//   - every tile reads the field as it was when the share began (the staging
//     reads a snapshot; the passes store into the live field);
//   - inside a tile, every thread of a phase reads the shared cells as they
//     were before the phase: each thread runs on its own copy of the stage
//     and its changes are merged, and two threads changing one cell is an
//     error;
//   - the stage is exactly the kernel's size (K*n*n*row stride + 2*n*n
//     doubles) with guard cells on both sides, and the field and its snapshot
//     have guards too: a guard that changes is an error;
//   - the live field starts every share as NaN; points the share does not
//     store take their snapshot value afterwards, so a point the share
//     should change but does not store stays wrong.
// The result must equal the oracle bit for bit.
//
// The message-mode step (xtile_steps.cuh: xdescribe, xcopies, xxpass, xyzpass) has its
// own replay, xtile_emulate: every share first packs the 26 messages of
// every rank on the host (region order of geom.cuh), then replays the tiles
// under the same model.  The tile records' addresses must lie in the field
// (the rank's own columns and ends) or in the messages (received ones);
// own addresses are moved from the snapshot to the live field, so the passes
// store into the live field, and the messages must come out unchanged.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <limits>
#include <string>
#include <vector>

#include "geom.cuh"
#include "ptile_steps.cuh"
#include "rows_setup.cuh"
#include "tables.h"
#include "tile_ops.cuh"
#include "pack_steps.cuh"
#include "xtile_steps.cuh"

using namespace faces;

namespace {

constexpr long kGuard = 64;
constexpr double kSentinel = -12345.678;

struct Err {
  std::string msg;
  bool ok = true;
  void set(const char *what, long tile)
  {
    if (!ok) return;
    char buf[256];
    snprintf(buf, sizeof(buf), "%s (tile %ld)", what, tile);
    msg = buf;
    ok = false;
  }
};

// the live field starts a share as NaN: a point a tile changes that was
// not NaN before the tile has been written twice in the share
void written_once(const std::vector<double> &before, const double *live, long total, Err &e, long tile)
{
  for (long i = 0; i < total && e.ok; i++)
    if (std::memcmp(&before[i], live + i, sizeof(double)) != 0 && !std::isnan(before[i]))
      e.set("a field point written twice in one share", tile);
}

bool guards_intact(const std::vector<double> &v, long inner)
{
  for (long i = 0; i < kGuard; i++)
    if (v[i] != kSentinel || v[kGuard + inner + i] != kSentinel) return false;
  return true;
}

// one phase of T threads under the model: thread t runs fn(stage copy, t);
// the cells it changes are applied to the stage afterwards
template <class F>
void phase(std::vector<double> &sm, int T, F fn, Err &e, long tile)
{
  const std::vector<double> before(sm);
  std::vector<int> owner(sm.size(), -1);
  std::vector<double> work;
  for (int t = 0; t < T; t++) {
    work = before;
    fn(work.data() + kGuard, t);
    for (size_t j = 0; j < sm.size(); j++) {
      if (std::memcmp(&work[j], &before[j], sizeof(double)) == 0) continue;
      if (owner[j] >= 0) { e.set("a stage cell changed by two threads of one phase", tile); return; }
      owner[j] = t;
      sm[j] = work[j];
    }
  }
}

template <int N, int K, int T>
int replay(FieldDesc f, double *live, double *snap, long total, const RowPlan &p, Err &e)
{
  constexpr int stage = tile_stage_size<N, K>();
  const long ncol = p.ntiles / p.nchunks;
  FieldDesc fs = f;
  fs.u = snap;  // the staging reads the share's starting field
  std::vector<double> sm(stage + 2 * kGuard, kSentinel);
  for (long tile = 0; tile < p.ntiles && e.ok; tile++) {
    TileCursor u;
    u.c = (int)(tile / ncol);
    const long col = tile - (long)u.c * ncol, t2 = col / p.ty;
    u.jy = (int)(col - t2 * p.ty);
    u.jz = (int)(t2 % p.tz);
    u.r = (int)(t2 / p.tz);
    std::fill(sm.begin(), sm.end(), kSentinel);
    std::fill(sm.begin() + kGuard, sm.end() - kGuard, std::numeric_limits<double>::quiet_NaN());
    PMeta meta{};
    int4 tinfo = make_int4(0, 0, 0, 0);
    for (int t = 0; t < T; t++) ptile::pstage<N, K, T>(fs, p, u, sm.data() + kGuard, &meta, &tinfo, t);
    if (meta.u != snap) { e.set("tile meta names another field", tile); break; }
    const int nk = tinfo.y;
    if (nk < 1 || nk > K || tinfo.x != u.c * p.chunk) { e.set("tile info out of range", tile); break; }
    const std::vector<double> before(live, live + total);
    phase(sm, T, [&](double *buf, int t) { ptile::pxpass<N, K, T>(live, buf, &meta, nk, t); }, e, tile);
    phase(sm, T, [&](double *buf, int t) { ptile::pyzpass<N, K, T>(live, buf, &meta, nk, t); }, e, tile);
    written_once(before, live, total, e, tile);
    if (!guards_intact(sm, stage)) e.set("stage guard cells changed", tile);
  }
  (void)total;
  return e.ok ? 0 : -1;
}

using ReplayFn = int (*)(FieldDesc, double *, double *, long, const RowPlan &, Err &);

template <int N, int K>
ReplayFn pick_t(int T)
{
  return T == 32 ? replay<N, K, 32> : replay<N, K, 256>;
}

template <int N>
ReplayFn pick_k(int K, int T)
{
  switch (K) {
    case 1: return pick_t<N, 1>(T);
    case 2: return pick_t<N, 2>(T);
    case 3: return pick_t<N, 3>(T);
    case 4: return pick_t<N, 4>(T);
    case 5: return pick_t<N, 5>(T);
    case 6: return pick_t<N, 6>(T);
    case 8: return pick_t<N, 8>(T);
    case 9: return pick_t<N, 9>(T);
    case 10: return pick_t<N, 10>(T);
    case 12: return pick_t<N, 12>(T);
    case 16: return pick_t<N, 16>(T);
    case 17: return pick_t<N, 17>(T);
    case 18: return pick_t<N, 18>(T);
    case 27: return pick_t<N, 27>(T);
    case 32: return pick_t<N, 32>(T);
    default: return nullptr;
  }
}

ReplayFn pick(int n, int K, int T)
{
  switch (n) {
    case 2: return pick_k<2>(K, T);
    case 3: return pick_k<3>(K, T);
    case 4: return pick_k<4>(K, T);
    case 5: return pick_k<5>(K, T);
    case 6: return pick_k<6>(K, T);
    case 7: return pick_k<7>(K, T);
    case 8: return pick_k<8>(K, T);
    case 9: return pick_k<9>(K, T);
    case 10: return pick_k<10>(K, T);
    case 11: return pick_k<11>(K, T);
    case 12: return pick_k<12>(K, T);
    default: return nullptr;
  }
}

}  // namespace

// nsteps shares of the periodic direct-mode field u (lx*ly*lz ranks of
// mx*my*mz elements of n^3 points, the device layout) with tiles of K
// elements and teams of T threads.  Returns 0, or -1 with a message in err.
extern "C" int ptile_emulate(int lx, int ly, int lz, int mx, int my, int mz, int n, int K, int T, double *u,
                             int nsteps, char *err, int errlen)
{
  Err e;
  tiledev::host_misaligned_copies() = 0;
  const ReplayFn fn = pick(n, K, T);
  if (!fn || (T != 32 && T != 256)) {
    snprintf(err, errlen, "no replay for n = %d, K = %d, T = %d", n, K, T);
    return -1;
  }
  FieldDesc f{};
  f.n = n;
  f.m[0] = mx; f.m[1] = my; f.m[2] = mz;
  f.L[0] = lx; f.L[1] = ly; f.L[2] = lz;
  f.periodic = 1;
  f.mode = kDirect;
  f.nranks = lx * ly * lz;
  f.sjy = (long)n * n * n * mx;
  f.sjz = jz_stride(n, mx, my);
  f.R = f.sjz * mz;
  const long total = f.R * f.nranks;
  std::vector<int> nbr = neighbour_table(f.L, true);
  std::vector<long> off(nbr.size(), -1);
  f.nbr = nbr.data();
  f.msg_off = off.data();
  f.recv_off = off.data();
  f.msg = nullptr;
  std::vector<double> live(total + 2 * kGuard, kSentinel), snap(total + 2 * kGuard, kSentinel);
  f.u = live.data() + kGuard;
  RowPlan p = make_row_plan(f, K, 0);
  if (p.chunk != K && K <= mx) {
    snprintf(err, errlen, "plan chunk %d for K = %d", p.chunk, K);
    return -1;
  }
  for (int step = 0; step < nsteps && e.ok; step++) {
    std::memcpy(snap.data() + kGuard, u, sizeof(double) * total);
    std::fill(live.begin() + kGuard, live.end() - kGuard, std::numeric_limits<double>::quiet_NaN());
    fn(f, live.data() + kGuard, snap.data() + kGuard, total, p, e);
    if (e.ok && (!guards_intact(live, total) || !guards_intact(snap, total))) e.set("field guard cells changed", -1);
    if (e.ok && tiledev::host_misaligned_copies() != 0) e.set("a 16-byte copy from or to an address not 16-byte aligned", -1);
    for (long i = 0; i < total && e.ok; i++) {
      const double v = live[kGuard + i];
      u[i] = std::isnan(v) ? snap[kGuard + i] : v;
    }
  }
  if (!e.ok) {
    snprintf(err, errlen, "%s", e.msg.c_str());
    return -1;
  }
  return 0;
}

namespace {

// the 26 messages of every rank from field u: message (r, dir) holds
// region(dir) of rank r in region_pos order
void host_pack(const FieldDesc &f, const double *u, double *msg, const std::vector<long> &off)
{
  const int n = f.n;
  for (int r = 0; r < f.nranks; r++)
    for (int dir = 0; dir < 27; dir++) {
      if (dir == 13 || off[r * 27 + dir] < 0) continue;
      const int d[3] = {dir % 3 - 1, (dir / 3) % 3 - 1, dir / 9 - 1};
      double *out = msg + off[r * 27 + dir];
      int i[3], j[3];
      for (j[2] = 0; j[2] < f.m[2]; j[2]++)
        for (j[1] = 0; j[1] < f.m[1]; j[1]++)
          for (j[0] = 0; j[0] < f.m[0]; j[0]++)
            for (i[2] = 0; i[2] < n; i[2]++)
              for (i[1] = 0; i[1] < n; i[1]++)
                for (i[0] = 0; i[0] < n; i[0]++) {
                  bool in = true;
                  for (int a = 0; a < 3; a++) {
                    if (d[a] < 0) in = in && i[a] == 0 && j[a] == 0;
                    if (d[a] > 0) in = in && i[a] == n - 1 && j[a] == f.m[a] - 1;
                  }
                  if (!in) continue;
                  out[region_pos(f, d, i, j)] = u[(long)r * f.R + elem_index(f, i[0], i[1], i[2], j[0], j[1], j[2])];
                }
    }
}

template <int N, int K, int T, bool OPEN>
int xreplay(FieldDesc f, double *live, double *snap, long total, double *msg, long msg_total, const RowPlan &p,
            const std::vector<char> &packread, Err &e)
{
  constexpr int stage = tile_stage_size<N, K>();
  const long ncol = p.ntiles / p.nchunks;
  FieldDesc fs = f;
  fs.u = snap;
  auto in = [](const double *q, const double *b, long len) { return b && q >= b && q < b + len; };
  std::vector<double> sm(stage + 2 * kGuard, kSentinel);
  for (long tile = 0; tile < p.ntiles && e.ok; tile++) {
    TileCursor u;
    u.c = (int)(tile / ncol);
    const long col = tile - (long)u.c * ncol, t2 = col / p.ty;
    u.jy = (int)(col - t2 * p.ty);
    u.jz = (int)(t2 % p.tz);
    u.r = (int)(t2 / p.tz);
    std::fill(sm.begin(), sm.end(), kSentinel);
    std::fill(sm.begin() + kGuard, sm.end() - kGuard, std::numeric_limits<double>::quiet_NaN());
    XMeta meta{};
    for (int t = 0; t < T; t++) xtile::xdescribe<N, OPEN, T>(fs, p, u, &meta, t);
    const int nk = meta.nk;
    if (nk < 1 || nk > K || meta.jx0 != u.c * p.chunk) { e.set("tile record out of range", tile); break; }
    const bool hx = (meta.flags & 1) != 0;
    for (int t = 0; t < T; t++) xtile::xcopies<N, K, OPEN, T>(&meta, sm.data() + kGuard, t);
    // own addresses point into the snapshot: move them to the live field;
    // received ones must lie in the messages and are never written; absent
    // ones (open fields) are null, and every one exists in a periodic field
    for (int sidx = 0; sidx < 4 && e.ok; sidx++) {
      double **ps[3] = {&meta.col[sidx], &meta.lo[sidx], &meta.hi[sidx]};
      const int own[3] = {(meta.wcol >> sidx) & 1, (meta.wlo >> sidx) & 1, 0};
      for (int q = 0; q < 3; q++) {
        double *a = *ps[q];
        if (q == 2 && !hx) {
          if (a) { e.set("an upper end on a chunk that is not the last", tile); break; }
          continue;
        }
        if (!a) {
          if (!OPEN) { e.set("an absent column or end in a periodic field", tile); break; }
          if (own[q]) { e.set("an absent column or end marked as own", tile); break; }
          continue;
        }
        if (in(a, snap, total)) {
          if (!own[q]) { e.set("a column or end in the field not marked as own", tile); break; }
          *ps[q] = live + (a - snap);
        } else if (!in(a, msg, msg_total) || own[q]) {
          e.set("tile record address outside the field and messages", tile);
          break;
        }
      }
    }
    if (!e.ok) break;
    const std::vector<double> before(live, live + total);
    // the kernel's choice: complete tiles take the passes' periodic form
    if (xtile::complete<OPEN>(&meta)) {
      phase(sm, T, [&](double *buf, int t) { xtile::xxpass<N, K, false, T>(buf, &meta, t); }, e, tile);
      phase(sm, T, [&](double *buf, int t) { xtile::xyzpass<N, K, false, T>(buf, &meta, t); }, e, tile);
    } else {
      phase(sm, T, [&](double *buf, int t) { xtile::xxpass<N, K, OPEN, T>(buf, &meta, t); }, e, tile);
      phase(sm, T, [&](double *buf, int t) { xtile::xyzpass<N, K, OPEN, T>(buf, &meta, t); }, e, tile);
    }
    written_once(before, live, total, e, tile);
    if (!guards_intact(sm, stage)) e.set("stage guard cells changed", tile);
    // the fused pack: an interior tile runs beside the other blocks' packing,
    // so it may change no point the pack reads (its record holds no message:
    // every address in it is marked own, checked above)
    if (!packread.empty() && xtile::interior(&meta))
      for (long i = 0; i < total && e.ok; i++)
        if (packread[i] && std::memcmp(&before[i], live + i, sizeof(double)) != 0)
          e.set("an interior tile changed a point the pack reads", tile);
  }
  return e.ok ? 0 : -1;
}

using XReplayFn = int (*)(FieldDesc, double *, double *, long, double *, long, const RowPlan &,
                          const std::vector<char> &, Err &);

template <int N, int K>
XReplayFn xpick_t(int T, bool open)
{
  if (open) return T == 32 ? xreplay<N, K, 32, true> : xreplay<N, K, 256, true>;
  return T == 32 ? xreplay<N, K, 32, false> : xreplay<N, K, 256, false>;
}

template <int N>
XReplayFn xpick_k(int K, int T, bool open)
{
  switch (K) {
    case 1: return xpick_t<N, 1>(T, open);
    case 2: return xpick_t<N, 2>(T, open);
    case 4: return xpick_t<N, 4>(T, open);
    case 8: return xpick_t<N, 8>(T, open);
    case 16: return xpick_t<N, 16>(T, open);
    case 32: return xpick_t<N, 32>(T, open);
    default: return nullptr;
  }
}

XReplayFn xpick(int n, int K, int T, bool open)
{
  switch (n) {
    case 2: return xpick_k<2>(K, T, open);
    case 3: return xpick_k<3>(K, T, open);
    case 4: return xpick_k<4>(K, T, open);
    case 5: return xpick_k<5>(K, T, open);
    case 6: return xpick_k<6>(K, T, open);
    case 7: return xpick_k<7>(K, T, open);
    case 8: return xpick_k<8>(K, T, open);
    case 9: return xpick_k<9>(K, T, open);
    case 10: return xpick_k<10>(K, T, open);
    case 11: return xpick_k<11>(K, T, open);
    case 12: return xpick_k<12>(K, T, open);
    default: return nullptr;
  }
}

}  // namespace

// nsteps shares of the field u (the device layout) by the message-mode
// tile step, with tiles of K elements (the chunk) and teams of T threads:
// periodic or open, v-26 message mode or (one open rank) direct mode.
// Returns 0, or -1 with a message in err.
extern "C" int xtile_emulate(int lx, int ly, int lz, int mx, int my, int mz, int n, int K, int T, int periodic,
                             int messages, double *u, int nsteps, char *err, int errlen)
{
  Err e;
  tiledev::host_misaligned_copies() = 0;
  const XReplayFn fn = xpick(n, K, T, !periodic);
  if (!fn || (T != 32 && T != 256)) {
    snprintf(err, errlen, "no replay for n = %d, K = %d, T = %d", n, K, T);
    return -1;
  }
  FieldDesc f{};
  f.n = n;
  f.m[0] = mx; f.m[1] = my; f.m[2] = mz;
  f.L[0] = lx; f.L[1] = ly; f.L[2] = lz;
  f.periodic = periodic ? 1 : 0;
  f.mode = messages ? kMessages : kDirect;
  f.nranks = lx * ly * lz;
  f.sjy = (long)n * n * n * mx;
  f.sjz = jz_stride(n, mx, my);
  f.R = f.sjz * mz;
  if (!xtile_field(f)) {
    snprintf(err, errlen, "the message-mode step does not take this field");
    return -1;
  }
  const long total = f.R * f.nranks;
  std::vector<int> nbr = neighbour_table(f.L, periodic != 0);
  std::vector<long> off(nbr.size(), -1);
  const long msg_total = messages ? message_offsets(f, nbr, off) : 0;
  std::vector<long> roff = receive_offsets(nbr, off);
  f.nbr = nbr.data();
  f.msg_off = off.data();
  f.recv_off = roff.data();
  std::vector<double> msg(msg_total + 2 * kGuard, kSentinel), msg_copy;
  f.msg = msg.data() + kGuard;
  std::vector<double> live(total + 2 * kGuard, kSentinel), snap(total + 2 * kGuard, kSentinel);
  f.u = live.data() + kGuard;
  RowPlan p = make_row_plan(f, K, 0);
  if (p.chunk != K && K <= mx) {
    snprintf(err, errlen, "plan chunk %d for K = %d", p.chunk, K);
    return -1;
  }
  for (int step = 0; step < nsteps && e.ok; step++) {
    std::memcpy(snap.data() + kGuard, u, sizeof(double) * total);
    std::fill(msg.begin() + kGuard, msg.end() - kGuard, std::numeric_limits<double>::quiet_NaN());
    host_pack(f, u, msg.data() + kGuard, off);
    // the device pack (pack_steps.cuh, the fused kernel's prologue) on every
    // block of its grid: the same messages, and the points it reads
    std::vector<char> packread;
    if (messages) {
      packread.assign(total, 0);
      std::vector<double> msg2(msg_total, std::numeric_limits<double>::quiet_NaN());
      FieldDesc fp = f;
      fp.u = u;
      fp.msg = msg2.data();
      const PackGrid g = pack_grid(fp);
      auto touch = [&](const double *q) {
        const long i = (long)(q - u);
        if (i < 0 || i >= total) e.set("the pack reads outside the field", -1);
        else packread[i] = 1;
      };
      for (int by = 0; by < g.gy && e.ok; by++)
        for (int bx = 0; bx < g.gx; bx++)
          for (int t = 0; t < 256; t++) {
            if (g.wide) pack_block<unsigned long>(fp, by, bx, g.gx, t, 256, touch);
            else pack_block<unsigned>(fp, by, bx, g.gx, t, 256, touch);
          }
      if (e.ok && std::memcmp(msg2.data(), msg.data() + kGuard, sizeof(double) * msg_total) != 0)
        e.set("the device pack's messages differ from the host pack's", -1);
    }
    msg_copy = msg;
    std::fill(live.begin() + kGuard, live.end() - kGuard, std::numeric_limits<double>::quiet_NaN());
    fn(f, live.data() + kGuard, snap.data() + kGuard, total, msg.data() + kGuard, msg_total, p, packread, e);
    if (e.ok && (!guards_intact(live, total) || !guards_intact(snap, total))) e.set("field guard cells changed", -1);
    if (e.ok && tiledev::host_misaligned_copies() != 0) e.set("a 16-byte copy from or to an address not 16-byte aligned", -1);
    if (e.ok && std::memcmp(msg.data(), msg_copy.data(), sizeof(double) * msg.size()) != 0)
      e.set("the step changed a message", -1);
    for (long i = 0; i < total && e.ok; i++) {
      const double v = live[kGuard + i];
      u[i] = std::isnan(v) ? snap[kGuard + i] : v;
    }
  }
  if (!e.ok) {
    snprintf(err, errlen, "%s", e.msg.c_str());
    return -1;
  }
  return 0;
}

// ---------------------------------------------------------------------------
// v-6, basic and fused (v6_steps.cuh): every launch's thread bodies run for
// every thread index on the host, once in order and once in reverse order on
// a copy (threads of one launch touch disjoint cells, so the two must agree
// bit for bit); the message buffer starts each share as NaN between guard
// cells, so a message read before it is packed poisons the result.
// ---------------------------------------------------------------------------

#include "v6_steps.cuh"

namespace {

template <class F>
void launch_both_orders(long nthreads, double *u, long total, double *msg, long mtotal, F body, Err &e)
{
  std::vector<double> u2(u, u + total), m2(msg, msg + mtotal);
  for (long t = 0; t < nthreads; t++) body(u, msg, t);
  for (long t = nthreads - 1; t >= 0; t--) body(u2.data(), m2.data(), t);
  if (std::memcmp(u2.data(), u, sizeof(double) * total) || std::memcmp(m2.data(), msg, sizeof(double) * mtotal))
    e.set("a launch's result depends on the order of its threads", -1);
}

}  // namespace

extern "C" int v6_emulate(int lx, int ly, int lz, int mx, int my, int mz, int n, int periodic, int fused, int compute,
                          double *u, int nsteps, char *err, int errlen)
{
  Err e;
  FieldDesc f{};
  f.n = n;
  f.m[0] = mx; f.m[1] = my; f.m[2] = mz;
  f.L[0] = lx; f.L[1] = ly; f.L[2] = lz;
  f.periodic = periodic;
  f.mode = kDirect;
  f.nranks = lx * ly * lz;
  f.sjy = (long)n * n * n * mx;
  f.sjz = jz_stride(n, mx, my);
  f.R = f.sjz * mz;
  const long total = f.R * f.nranks;
  std::vector<int> nbr = neighbour_table(f.L, periodic != 0);
  f.nbr = nbr.data();
  const V6Geoms gs = v6_geoms(f);
  const long mtotal = gs.g[0].per_rank * f.nranks;
  std::vector<double> field(total + 2 * kGuard, kSentinel), msg(mtotal + 2 * kGuard, kSentinel);
  double *fu = field.data() + kGuard, *fm = msg.data() + kGuard;
  std::memcpy(fu, u, sizeof(double) * total);
  for (int step = 0; step < nsteps && e.ok; step++) {
    std::fill(msg.begin() + kGuard, msg.end() - kGuard, std::numeric_limits<double>::quiet_NaN());
    auto with = [&](double *uu) {
      FieldDesc g = f;
      g.u = uu;
      return g;
    };
    if (!fused) {
      for (int d = 2; d >= 0 && e.ok; d--) {
        const V6Geom &g = gs.g[d];
        launch_both_orders(f.nranks * 2 * g.F, fu, total, fm, mtotal,
                           [&](double *uu, double *mm, long t) { v6_pack_item<long>(with(uu), g, mm, t); }, e);
        launch_both_orders((long)f.nranks * f.m[0] * f.m[1] * f.m[2] * n * n, fu, total, fm, mtotal,
                           [&](double *uu, double *mm, long t) { v6_part_item<long>(with(uu), g, mm, compute, t); }, e);
      }
    } else {
      launch_both_orders(mtotal, fu, total, fm, mtotal,
                         [&](double *uu, double *mm, long t) { v6_early_item<long>(with(uu), gs, mm, t); }, e);
      for (int d = 2; d >= 1 && e.ok; d--)
        launch_both_orders((long)f.nranks * f.m[0] * f.m[1] * f.m[2] * n * n, fu, total, fm, mtotal,
                           [&](double *uu, double *mm, long t) {
                             v6_part_pack_item<long>(with(uu), gs, d, mm, compute, t);
                           },
                           e);
      launch_both_orders((long)f.nranks * f.m[0] * f.m[1] * f.m[2] * n * n, fu, total, fm, mtotal,
                         [&](double *uu, double *mm, long t) { v6_part_item<long>(with(uu), gs.g[0], mm, compute, t); },
                         e);
    }
    if (!guards_intact(field, total) || !guards_intact(msg, mtotal)) e.set("guard cells changed", -1);
  }
  std::memcpy(u, fu, sizeof(double) * total);
  if (!e.ok) {
    snprintf(err, errlen, "%s", e.msg.c_str());
    return -1;
  }
  return 0;
}

// ---------------------------------------------------------------------------
// The seam step (seam_steps.cuh): every slot of every chunk, then every item
// of the open upper boundary planes, run one by one.  The kernel has no
// barrier, so its threads may run in any order and at once: each point may be
// read and written by one thread of a share at most (every touched address is
// recorded with its thread), and every address must lie in the field.
// ---------------------------------------------------------------------------

#include "seam_steps.cuh"

namespace {

// the lean form: the lean kernel's items, then the boundary planes' (each
// launch in order or in reverse); one thread per item
template <int N, class T>
void seam_lean_share(const FieldDesc &f, bool reverse, long &who, T touch, Err &e)
{
  const int cols = f.nranks * f.m[1] * f.m[2], per = f.m[0] * seam_lean_slots(N);
  const long items = (long)cols * per;
  const long planes = f.periodic ? 0 : (long)f.nranks * seam_plane_items(f);
  for (long k = 0; k < items && e.ok; k++) {
    const long g = reverse ? items - 1 - k : k;
    who = g;
    seam_lean_item<N>(f, (int)(g / per), (int)(g % per), touch);
  }
  for (long k = 0; k < planes && e.ok; k++) {
    const long g = reverse ? planes - 1 - k : k;
    who = items + g;
    seam_plane_point(f, g, touch);
  }
}

template <int N>
void seam_share(const FieldDesc &f, int E, bool reverse, bool lean, Err &e)
{
  constexpr int S = seam_slots(N);
  const long total = f.R * f.nranks;
  const int nch = (f.m[0] + E - 1) / E;
  const long units = (long)f.nranks * f.m[2] * f.m[1] * nch;
  const long planes = f.periodic ? 0 : (long)f.nranks * seam_plane_items(f);
  std::vector<long> owner(total, -1);
  long who = 0;
  auto touch = [&](const double *p) {
    const long i = (long)(p - f.u);
    if (i < 0 || i >= total) { e.set("an address outside the field", who); return; }
    if (owner[i] >= 0 && owner[i] != who) { e.set("a point touched by two threads of one share", who); return; }
    owner[i] = who;
  };
  if (lean) {
    seam_lean_share<N>(f, reverse, who, touch, e);
    return;
  }
  // the kernel's loop: thread t of a 256-thread block takes slots t, t+256,
  // ... of each chunk; who = (chunk, thread)
  constexpr int T = 256;
  const long threads = units * T;
  for (long k = 0; k < threads + planes && e.ok; k++) {
    const long id = reverse ? threads + planes - 1 - k : k;
    who = id;
    if (id < threads) {
      const long w = id / T;
      const int t = (int)(id - w * T);
      const SeamUnit un = seam_unit(f, E, nch, w);
      const SeamChunk c = seam_chunk<N>(f, un.r, un.jy, un.jz, un.jx0, un.nk);
      const int items = un.nk * S;
      for (int q = t; q < items; q += T) seam_item<N>(f.u, c, q, touch);
    } else {
      seam_plane_point(f, id - threads, touch);
    }
  }
}

}  // namespace

extern "C" int seam_emulate(int lx, int ly, int lz, int mx, int my, int mz, int n, int periodic, int E, int mode,
                            double *u, int nsteps, char *err, int errlen)
{
  Err e;
  FieldDesc f{};
  f.n = n;
  f.m[0] = mx; f.m[1] = my; f.m[2] = mz;
  f.L[0] = lx; f.L[1] = ly; f.L[2] = lz;
  f.periodic = periodic;
  f.mode = kDirect;
  f.nranks = lx * ly * lz;
  f.sjy = (long)n * n * n * mx;
  f.sjz = jz_stride(n, mx, my);
  f.R = f.sjz * mz;
  const long total = f.R * f.nranks;
  std::vector<int> nbr = neighbour_table(f.L, periodic != 0);
  f.nbr = nbr.data();
  std::vector<double> field(total + 2 * kGuard, kSentinel);
  f.u = field.data() + kGuard;
  std::memcpy(f.u, u, sizeof(double) * total);
  if (E < 1 || E > mx) E = mx;
  for (int step = 0; step < nsteps && e.ok; step++) {
    switch (n) {
      case 2: seam_share<2>(f, E, (mode & 1) != 0, (mode & 2) != 0, e); break;
      case 3: seam_share<3>(f, E, (mode & 1) != 0, (mode & 2) != 0, e); break;
      case 4: seam_share<4>(f, E, (mode & 1) != 0, (mode & 2) != 0, e); break;
      case 5: seam_share<5>(f, E, (mode & 1) != 0, (mode & 2) != 0, e); break;
      case 6: seam_share<6>(f, E, (mode & 1) != 0, (mode & 2) != 0, e); break;
      case 7: seam_share<7>(f, E, (mode & 1) != 0, (mode & 2) != 0, e); break;
      case 8: seam_share<8>(f, E, (mode & 1) != 0, (mode & 2) != 0, e); break;
      case 9: seam_share<9>(f, E, (mode & 1) != 0, (mode & 2) != 0, e); break;
      case 10: seam_share<10>(f, E, (mode & 1) != 0, (mode & 2) != 0, e); break;
      case 11: seam_share<11>(f, E, (mode & 1) != 0, (mode & 2) != 0, e); break;
      case 12: seam_share<12>(f, E, (mode & 1) != 0, (mode & 2) != 0, e); break;
      case 16: seam_share<16>(f, E, (mode & 1) != 0, (mode & 2) != 0, e); break;
      default: e.set("n not replayed", -1);
    }
    if (!guards_intact(field, total)) e.set("guard cells changed", -1);
  }
  std::memcpy(u, f.u, sizeof(double) * total);
  if (!e.ok) {
    snprintf(err, errlen, "%s", e.msg.c_str());
    return -1;
  }
  return 0;
}
