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
    phase(sm, T, [&](double *buf, int t) { ptile::pxpass<N, K, T>(live, buf, &meta, nk, t); }, e, tile);
    phase(sm, T, [&](double *buf, int t) { ptile::pyzpass<N, K, T>(live, buf, &meta, nk, t); }, e, tile);
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
    case 6: return pick_t<N, 6>(T);
    case 8: return pick_t<N, 8>(T);
    case 9: return pick_t<N, 9>(T);
    case 16: return pick_t<N, 16>(T);
    case 17: return pick_t<N, 17>(T);
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
