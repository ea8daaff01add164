/*
 * faces_oracle.c -- CPU oracle for the Faces halo-sum step (test
 * infrastructure only; see faces_oracle.h for the contract and layout).
 *
 * Compile with -ffp-contract=off: every sum below must round once per add on
 * every host (aarch64 gcc fuses a*b+c by default, which would change the
 * reference init values).
 */
#include "faces_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* ------------------------------------------------------------------ */
/* geometry                                                             */
/* ------------------------------------------------------------------ */

typedef struct geo {
  int n, m[3], L[3], periodic, nranks;
  long s[6];  /* strides of ix, iy, iz, jx, jy, jz */
  long R;     /* doubles per rank */
} geo;

int orc_check(const orc_geom *g)
{
  if (!g) return -1;
  if (g->n < 2) return -2;
  if (g->lx < 1 || g->ly < 1 || g->lz < 1) return -3;
  if (g->mx < 1 || g->my < 1 || g->mz < 1) return -4;
  return 0;
}

long orc_jz_stride(const orc_geom *g)
{
  /* DArray page padding of the second-to-last stride (gpu/DArray.h:91-101) */
  const long page = 4096 / (long)sizeof(double);
  const long s4 = (long)g->n * g->n * g->n * g->mx * g->my;
  return ((s4 - 1) / page + 1) * page;
}

long orc_rank_doubles(const orc_geom *g) { return orc_jz_stride(g) * g->mz; }

long orc_total_doubles(const orc_geom *g)
{
  return orc_rank_doubles(g) * g->lx * g->ly * g->lz;
}

static void geo_make(const orc_geom *g, geo *o)
{
  o->n = g->n;
  o->m[0] = g->mx; o->m[1] = g->my; o->m[2] = g->mz;
  o->L[0] = g->lx; o->L[1] = g->ly; o->L[2] = g->lz;
  o->periodic = g->periodic;
  o->nranks = g->lx * g->ly * g->lz;
  const long n = g->n;
  o->s[0] = 1;
  o->s[1] = n;
  o->s[2] = n * n;
  o->s[3] = n * n * n;
  o->s[4] = n * n * n * g->mx;
  o->s[5] = orc_jz_stride(g);
  o->R = orc_rank_doubles(g);
}

static inline long gidx(const geo *o, const int i[3], const int j[3])
{
  return i[0] * o->s[0] + i[1] * o->s[1] + i[2] * o->s[2] +
         j[0] * o->s[3] + j[1] * o->s[4] + j[2] * o->s[5];
}

/* rank coordinates, gpu/Mugs.cc:23-25 */
static inline void rank_coords(const geo *o, int r, int k[3])
{
  k[2] = r / (o->L[0] * o->L[1]);
  k[1] = (r - k[2] * o->L[0] * o->L[1]) / o->L[0];
  k[0] = r - (k[2] * o->L[1] + k[1]) * o->L[0];
}

/* neighbor(dx,dy,dz), gpu/Mugs.cc:72-83; -1 plays MPI_PROC_NULL.  With
 * periodic=1 the coordinates wrap (the reference never wraps). */
static int neighbor(const geo *o, int r, const int d[3])
{
  int k[3];
  rank_coords(o, r, k);
  for (int a = 0; a < 3; a++) {
    int kk = k[a] + d[a];
    if (kk < 0 || kk >= o->L[a]) {
      if (!o->periodic) return -1;
      kk = (kk + o->L[a]) % o->L[a];
    }
    k[a] = kk;
  }
  return (k[2] * o->L[1] + k[1]) * o->L[0] + k[0];
}

int orc_max_threads(void)
{
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

/* ------------------------------------------------------------------ */
/* initial values                                                       */
/* ------------------------------------------------------------------ */

static inline uint64_t splitmix64(uint64_t x)
{
  /* Steele, Lea & Flood, "Fast splittable pseudorandom number generators" */
  uint64_t z = x + 0x9E3779B97F4A7C15ULL;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
}

double orc_int_value(uint64_t seed, long index)
{
  return (double)(splitmix64(seed * 0x9E3779B97F4A7C15ULL + (uint64_t)index) >> 44);
}

/* gpu/main.cc:18 (device init) and :30 (host ainit): the same formula. */
static inline double ref_value(int ix, int iy, int iz, int jx, int jy, int jz)
{
  const int whole = jz * 10000 + jy * 100 + jx;
  double v = (double)whole + iz * 0.01;
  v = v + iy * 0.0001;
  v = v + ix * 0.000001;
  return v;
}

void orc_init_ref(const orc_geom *g, double *u)
{
  geo o;
  geo_make(g, &o);
  memset(u, 0, sizeof(double) * o.R * o.nranks);
  const int n = o.n;
  for (int r = 0; r < o.nranks; r++) {
    double *ur = u + (long)r * o.R;
#pragma omp parallel for collapse(3)
    for (int jz = 0; jz < o.m[2]; jz++)
      for (int jy = 0; jy < o.m[1]; jy++)
        for (int jx = 0; jx < o.m[0]; jx++)
          for (int iz = 0; iz < n; iz++)
            for (int iy = 0; iy < n; iy++)
              for (int ix = 0; ix < n; ix++) {
                const int i[3] = {ix, iy, iz}, j[3] = {jx, jy, jz};
                ur[gidx(&o, i, j)] = ref_value(ix, iy, iz, jx, jy, jz);
              }
  }
}

void orc_init_int(const orc_geom *g, double *u, uint64_t seed)
{
  geo o;
  geo_make(g, &o);
  const int n = o.n;
  const long ne = (long)n * n * n * o.m[0] * o.m[1]; /* unpadded plane */
  for (int r = 0; r < o.nranks; r++) {
#pragma omp parallel for
    for (long jz = 0; jz < o.m[2]; jz++) {
      const long base = (long)r * o.R + jz * o.s[5];
      for (long p = 0; p < o.s[5]; p++)
        u[base + p] = (p < ne) ? orc_int_value(seed, base + p) : 0.0;
    }
  }
}

/* ------------------------------------------------------------------ */
/* tree sum over the copies of one shared point                          */
/* ------------------------------------------------------------------ */

/* Copies of one point along one dimension: cnt (1 or 2) pairs of (element,
 * point index); slot 0 is the lower element (index n-1), slot 1 the upper
 * element (index 0).  Elements may lie outside [0,m): then rank-crossing. */
typedef struct dcop {
  int cnt;
  int e[2];
  int i[2];
} dcop;

/* value pointers of the up-to-8 copies, c[bz][by][bx] */
typedef struct gcop {
  int cnt[3];
  double *p[2][2][2];
  const double *q[2][2][2]; /* read source (may differ from p: messages) */
} gcop;

/* The sum every copy receives: x pairs, then y pairs, then z pairs.  This is
 * the order Mugs::share's in-place passes produce (gpu/Mugs.cc:140-202). */
static inline double tree_sum(const gcop *c)
{
  double sy[2];
  for (int bz = 0; bz < c->cnt[2]; bz++) {
    double sx[2];
    for (int by = 0; by < c->cnt[1]; by++) {
      sx[by] = *c->q[bz][by][0];
      if (c->cnt[0] == 2) sx[by] = sx[by] + *c->q[bz][by][1];
    }
    sy[bz] = (c->cnt[1] == 2) ? sx[0] + sx[1] : sx[0];
  }
  return (c->cnt[2] == 2) ? sy[0] + sy[1] : sy[0];
}

/* ------------------------------------------------------------------ */
/* formulation 1: global-mesh groups                                     */
/* ------------------------------------------------------------------ */

/* Global point coordinate g along a dimension with M = L*m elements: element
 * E holds g = E*(n-1)+i.  A point with g % (n-1) == 0 lies on the seam
 * between elements E-1 and E. */
static void global_dim(long g, int M, int n, int periodic, dcop *d)
{
  const int nm1 = n - 1;
  const long E = g / nm1;
  const int i = (int)(g % nm1);
  if (i != 0) {
    d->cnt = 1; d->e[0] = (int)E; d->i[0] = i;
  } else if (periodic) {
    d->cnt = 2; d->e[0] = (int)((E - 1 + M) % M); d->i[0] = nm1; d->e[1] = (int)(E % M); d->i[1] = 0;
  } else if (E == 0) {
    d->cnt = 1; d->e[0] = 0; d->i[0] = 0;
  } else if (E == M) {
    d->cnt = 1; d->e[0] = M - 1; d->i[0] = nm1;
  } else {
    d->cnt = 2; d->e[0] = (int)E - 1; d->i[0] = nm1; d->e[1] = (int)E; d->i[1] = 0;
  }
}

static double *global_ptr(const geo *o, double *u, const int E[3], const int i[3])
{
  int k[3], j[3];
  for (int a = 0; a < 3; a++) { k[a] = E[a] / o->m[a]; j[a] = E[a] % o->m[a]; }
  const int r = (k[2] * o->L[1] + k[1]) * o->L[0] + k[0];
  return u + (long)r * o->R + gidx(o, i, j);
}

static void groups_step(const geo *o, double *u, int compute)
{
  const int n = o->n, nm1 = n - 1;
  long G[3], M[3], span[3];
  for (int a = 0; a < 3; a++) {
    M[a] = (long)o->L[a] * o->m[a];
    G[a] = M[a] * nm1 + (o->periodic ? 0 : 1);
    span[a] = (long)o->m[a] * nm1; /* points per rank subdomain */
  }
#pragma omp parallel for schedule(static)
  for (long gz = 0; gz < G[2]; gz++) {
    dcop dz, dy, dx;
    global_dim(gz, (int)M[2], n, o->periodic, &dz);
    for (long gy = 0; gy < G[1]; gy++) {
      global_dim(gy, (int)M[1], n, o->periodic, &dy);
      for (long gx = 0; gx < G[0]; gx++) {
        global_dim(gx, (int)M[0], n, o->periodic, &dx);
        if (dx.cnt * dy.cnt * dz.cnt == 1) continue;
        if (!compute && (gx % span[0]) && (gy % span[1]) && (gz % span[2])) continue;
        gcop c;
        c.cnt[0] = dx.cnt; c.cnt[1] = dy.cnt; c.cnt[2] = dz.cnt;
        for (int bz = 0; bz < dz.cnt; bz++)
          for (int by = 0; by < dy.cnt; by++)
            for (int bx = 0; bx < dx.cnt; bx++) {
              const int E[3] = {dx.e[bx], dy.e[by], dz.e[bz]};
              const int i[3] = {dx.i[bx], dy.i[by], dz.i[bz]};
              c.p[bz][by][bx] = global_ptr(o, u, E, i);
              c.q[bz][by][bx] = c.p[bz][by][bx];
            }
        const double s = tree_sum(&c);
        for (int bz = 0; bz < dz.cnt; bz++)
          for (int by = 0; by < dy.cnt; by++)
            for (int bx = 0; bx < dx.cnt; bx++) *c.p[bz][by][bx] = s;
      }
    }
  }
}

void orc_groups_share(const orc_geom *g, double *u, int compute, int nsteps)
{
  geo o;
  geo_make(g, &o);
  for (int t = 0; t < nsteps; t++) groups_step(&o, u, compute);
}

/* ------------------------------------------------------------------ */
/* 26 direction-keyed messages                                          */
/* ------------------------------------------------------------------ */

/* Direction index: dir = (dx+1) + 3*(dy+1) + 9*(dz+1), 13 = self (unused).
 * region(d) of a rank = its points on the subdomain boundary facing d: for
 * d_a = -1 the plane j_a = 0, i_a = 0; for d_a = +1 the plane j_a = m_a-1,
 * i_a = n-1; d_a = 0 leaves (i_a, j_a) free.  Messages list region(d) with
 * the free point indices fastest (x before y before z), then the free
 * element indices: the layout of the reference's zfs(ix,iy,jx,jy),
 * yfs(ix,iz,jx,jz), xfs(iy,iz,jy,jz), xes(ix,jx), ... buffers
 * (gpu/v-26-messages/Faces.cc:16-27). */
static inline void dir_vec(int dir, int d[3])
{
  d[0] = dir % 3 - 1;
  d[1] = (dir / 3) % 3 - 1;
  d[2] = dir / 9 - 1;
}

static inline int dir_index(const int d[3]) { return (d[0] + 1) + 3 * (d[1] + 1) + 9 * (d[2] + 1); }

static long region_size(const geo *o, const int d[3])
{
  long s = 1;
  for (int a = 0; a < 3; a++)
    if (d[a] == 0) s *= (long)o->n * o->m[a];
  return s;
}

/* position inside the message of the point (i,j) of region(d) */
static inline long region_pos(const geo *o, const int d[3], const int i[3], const int j[3])
{
  long pos = 0, mul = 1;
  for (int a = 0; a < 3; a++)
    if (d[a] == 0) { pos += i[a] * mul; mul *= o->n; }
  for (int a = 0; a < 3; a++)
    if (d[a] == 0) { pos += j[a] * mul; mul *= o->m[a]; }
  return pos;
}

/* inverse of region_pos */
static inline void region_point(const geo *o, const int d[3], long pos, int i[3], int j[3])
{
  for (int a = 0; a < 3; a++)
    if (d[a] != 0) {
      i[a] = d[a] < 0 ? 0 : o->n - 1;
      j[a] = d[a] < 0 ? 0 : o->m[a] - 1;
    }
  for (int a = 0; a < 3; a++)
    if (d[a] == 0) { i[a] = (int)(pos % o->n); pos /= o->n; }
  for (int a = 0; a < 3; a++)
    if (d[a] == 0) { j[a] = (int)(pos % o->m[a]); pos /= o->m[a]; }
}

typedef struct msgs {
  double *buf;      /* all send buffers */
  long *off;        /* off[r*27+dir] */
} msgs;

static void msgs_alloc(const geo *o, msgs *mb)
{
  mb->off = (long *)malloc(sizeof(long) * 27 * o->nranks);
  long tot = 0;
  for (int r = 0; r < o->nranks; r++)
    for (int dir = 0; dir < 27; dir++) {
      int d[3];
      dir_vec(dir, d);
      mb->off[r * 27 + dir] = tot;
      if (dir != 13) tot += region_size(o, d);
    }
  mb->buf = (double *)calloc((size_t)(tot > 0 ? tot : 1), sizeof(double));
}

static void msgs_free(msgs *mb)
{
  free(mb->buf);
  free(mb->off);
}

/* send buffer of rank r toward direction d: the raw values of region(d) */
static void pack_all(const geo *o, const double *u, msgs *mb)
{
  for (int r = 0; r < o->nranks; r++) {
    const double *ur = u + (long)r * o->R;
    for (int dir = 0; dir < 27; dir++) {
      if (dir == 13) continue;
      int d[3];
      dir_vec(dir, d);
      if (neighbor(o, r, d) < 0) continue;
      double *sb = mb->buf + mb->off[r * 27 + dir];
      const long sz = region_size(o, d);
#pragma omp parallel for schedule(static)
      for (long p = 0; p < sz; p++) {
        int i[3], j[3];
        region_point(o, d, p, i, j);
        sb[p] = ur[gidx(o, i, j)];
      }
    }
  }
}

/* the message rank r receives from direction d = what neighbor(r,d) sent
 * toward -d (direction-keyed: correct when one rank is the neighbour in
 * several directions, e.g. a periodic grid with l = 1 or 2) */
static const double *recv_buf(const geo *o, const msgs *mb, int r, const int d[3])
{
  const int q = neighbor(o, r, d);
  if (q < 0) return NULL;
  const int md[3] = {-d[0], -d[1], -d[2]};
  return mb->buf + mb->off[q * 27 + dir_index(md)];
}

/* ------------------------------------------------------------------ */
/* formulation 2: Mugs::share restated                                   */
/* ------------------------------------------------------------------ */

/* One in-place pair pass along dimension a (gpu/Mugs.cc:140-202): for every
 * pair of neighbouring elements (j_a-1, j_a) the copy at i_a = 0 of the upper
 * element becomes the sum of both copies and the lower copy (i_a = n-1) takes
 * that value.  With compute=0 only points on the subdomain boundary of one of
 * the other two dimensions are summed (gpu/Mugs.cc:146-150). */
static void mugs_pass(const geo *o, double *ur, int a, int compute)
{
  const int n = o->n, nm1 = n - 1;
  const int b = (a + 1) % 3, c = (a + 2) % 3;
  const long nb = (long)o->m[b] * n, nc = (long)o->m[c] * n;
#pragma omp parallel for collapse(2) schedule(static)
  for (long pc = 0; pc < nc; pc++)
    for (long pb = 0; pb < nb; pb++) {
      int i[3], j[3];
      j[c] = (int)(pc / n); i[c] = (int)(pc % n);
      j[b] = (int)(pb / n); i[b] = (int)(pb % n);
      if (!compute) {
        const int onb = (j[b] == 0 && i[b] == 0) || (j[b] == o->m[b] - 1 && i[b] == nm1);
        const int onc = (j[c] == 0 && i[c] == 0) || (j[c] == o->m[c] - 1 && i[c] == nm1);
        if (!onb && !onc) continue;
      }
      for (int ja = 1; ja < o->m[a]; ja++) {
        int ia[3] = {i[0], i[1], i[2]}, ja3[3] = {j[0], j[1], j[2]};
        ia[a] = 0; ja3[a] = ja;
        const long hi = gidx(o, ia, ja3);
        ia[a] = nm1; ja3[a] = ja - 1;
        const long lo = gidx(o, ia, ja3);
        ur[hi] = ur[hi] + ur[lo];
        ur[lo] = ur[hi];
      }
    }
}

/* Remote adds in the reference's order (gpu/Mugs.cc:337-412): x faces, y
 * faces, z faces, then edges along x, y, z, then the 8 corners.  Each local
 * point of region(d) adds the matching value the neighbour in direction d
 * sent. */
static void mugs_unpack(const geo *o, double *ur, int r, const msgs *mb)
{
  /* categories: faces by normal axis, edges by free axis, corners */
  for (int cat = 0; cat < 7; cat++) {
    for (int dir = 0; dir < 27; dir++) {
      if (dir == 13) continue;
      int d[3];
      dir_vec(dir, d);
      const int nz = (d[0] != 0) + (d[1] != 0) + (d[2] != 0);
      int want;
      if (nz == 1) want = (d[0] != 0) ? 0 : (d[1] != 0) ? 1 : 2;
      else if (nz == 2) want = 3 + ((d[0] == 0) ? 0 : (d[1] == 0) ? 1 : 2);
      else want = 6;
      if (want != cat) continue;
      const double *rb = recv_buf(o, mb, r, d);
      if (!rb) continue;
      const long sz = region_size(o, d);
#pragma omp parallel for schedule(static)
      for (long p = 0; p < sz; p++) {
        int i[3], j[3];
        region_point(o, d, p, i, j);
        const long k = gidx(o, i, j);
        ur[k] = ur[k] + rb[p];
      }
    }
  }
}

void orc_mugs_share(const orc_geom *g, double *u, int compute, int nsteps)
{
  geo o;
  geo_make(g, &o);
  msgs mb;
  msgs_alloc(&o, &mb);
  const int exchange = o.nranks > 1 || o.periodic; /* gpu/Mugs.cc:102,205 */
  for (int t = 0; t < nsteps; t++) {
    for (int r = 0; r < o.nranks; r++) {
      double *ur = u + (long)r * o.R;
      mugs_pass(&o, ur, 0, compute);
      mugs_pass(&o, ur, 1, compute);
      mugs_pass(&o, ur, 2, compute);
    }
    if (!exchange) continue;
    pack_all(&o, u, &mb);
    for (int r = 0; r < o.nranks; r++) mugs_unpack(&o, u + (long)r * o.R, r, &mb);
  }
  msgs_free(&mb);
}

/* ------------------------------------------------------------------ */
/* formulation 3: v-26 pack / inner / swap / unpack on the host           */
/* ------------------------------------------------------------------ */

/* Copies along one dimension of the rank-local point coordinate
 * g in [0, m*(n-1)]; elements -1 and m are the neighbours' (remote). */
static inline void local_dim(int g, int m, int n, dcop *d)
{
  const int nm1 = n - 1;
  const int E = g / nm1, i = g % nm1;
  if (i != 0) { d->cnt = 1; d->e[0] = E; d->i[0] = i; return; }
  d->cnt = 2; d->e[0] = E - 1; d->i[0] = nm1; d->e[1] = E; d->i[1] = 0;
}

/* Gather the copies of the rank-local point (gx,gy,gz): local copies point
 * into u, remote ones into the received messages.  Copies whose neighbour
 * does not exist are dropped.  Returns the number of copies. */
static int v26_gather(const geo *o, double *ur, int r, const msgs *mb, const int gp[3], gcop *c,
                      int *nlocal)
{
  dcop dd[3];
  for (int a = 0; a < 3; a++) local_dim(gp[a], o->m[a], o->n, &dd[a]);
  int keep[3][2], kcnt[3];
  /* a copy is dropped only if it lies outside the subdomain in a direction
   * with no neighbour; decide per dimension first */
  for (int a = 0; a < 3; a++) {
    kcnt[a] = 0;
    for (int b = 0; b < dd[a].cnt; b++) {
      const int e = dd[a].e[b];
      int dv[3] = {0, 0, 0};
      dv[a] = (e < 0) ? -1 : (e >= o->m[a]) ? 1 : 0;
      if (dv[a] != 0 && neighbor(o, r, dv) < 0) continue;
      keep[a][kcnt[a]++] = b;
    }
  }
  int nl = 0;
  for (int a = 0; a < 3; a++) c->cnt[a] = kcnt[a];
  for (int bz = 0; bz < kcnt[2]; bz++)
    for (int by = 0; by < kcnt[1]; by++)
      for (int bx = 0; bx < kcnt[0]; bx++) {
        const int sel[3] = {keep[0][bx], keep[1][by], keep[2][bz]};
        int d[3], i[3], j[3];
        for (int a = 0; a < 3; a++) {
          const int e = dd[a].e[sel[a]];
          i[a] = dd[a].i[sel[a]];
          d[a] = (e < 0) ? -1 : (e >= o->m[a]) ? 1 : 0;
          j[a] = (e < 0) ? o->m[a] - 1 : (e >= o->m[a]) ? 0 : e;
        }
        if (d[0] == 0 && d[1] == 0 && d[2] == 0) {
          c->p[bz][by][bx] = ur + gidx(o, i, j);
          c->q[bz][by][bx] = c->p[bz][by][bx];
          nl++;
        } else {
          /* remote copy: the neighbour in direction d sent region(-d); its
           * free coordinates equal ours */
          const int md[3] = {-d[0], -d[1], -d[2]};
          const double *rb = recv_buf(o, mb, r, d);
          c->p[bz][by][bx] = NULL;
          c->q[bz][by][bx] = rb + region_pos(o, md, i, j);
        }
      }
  *nlocal = nl;
  return kcnt[0] * kcnt[1] * kcnt[2];
}

static void v26_step(const geo *o, double *u, int compute, msgs *mb)
{
  const int nm1 = o->n - 1;
  int G[3];
  for (int a = 0; a < 3; a++) G[a] = o->m[a] * nm1; /* local g in [0, G] */

  /* pack (gpu/v-26-messages/Faces.cc:243-293): raw values, before any sum */
  pack_all(o, u, mb);

  for (int r = 0; r < o->nranks; r++) {
    double *ur = u + (long)r * o->R;
    /* inner (gpu/v-26-messages/Faces.cc:301-376): groups strictly inside the
     * subdomain; every copy is local */
    if (compute) {
      /* element loops as the reference's fused inner kernel: element
       * (jx,jy,jz) owns its points with i_a in [0, n-2] that lie on a seam
       * with a lower element (i_a = 0, j_a > 0); points on the subdomain
       * boundary (i_a = 0, j_a = 0) are left to the unpack */
      const int n = o->n;
      const long s3 = o->s[3], s4 = o->s[4], s5 = o->s[5];
      const long ox = -s3 + nm1, oy = -s4 + (long)nm1 * n, oz = -s5 + (long)nm1 * n * n;
#pragma omp parallel for collapse(2) schedule(static)
      for (int jz = 0; jz < o->m[2]; jz++)
        for (int jy = 0; jy < o->m[1]; jy++)
          for (int jx = 0; jx < o->m[0]; jx++) {
            double *e = ur + jx * s3 + jy * s4 + jz * s5;
            const int lx = jx > 0 ? 0 : 1, ly = jy > 0 ? 0 : 1, lz = jz > 0 ? 0 : 1;
            for (int iz = lz; iz < nm1; iz++)
              for (int iy = ly; iy < nm1; iy++) {
                /* a row with iy, iz off the seams only has its ix = 0 point */
                const int xend = (iy && iz) ? (lx == 0 ? 1 : 0) : nm1;
                for (int ix = lx; ix < xend; ix++) {
                  double *p = e + ix + (long)iy * n + (long)iz * n * n;
                  const int cx = ix == 0 ? 2 : 1, cy = iy == 0 ? 2 : 1, cz = iz == 0 ? 2 : 1;
                  double sy[2];
                  for (int bz = 0; bz < cz; bz++) {
                    double sx[2];
                    for (int by = 0; by < cy; by++) {
                      const double *q = p + (bz ? oz : 0) + (by ? oy : 0);
                      sx[by] = (cx == 2) ? q[0] + q[ox] : q[0];
                    }
                    sy[bz] = (cy == 2) ? sx[0] + sx[1] : sx[0];
                  }
                  const double s = (cz == 2) ? sy[0] + sy[1] : sy[0];
                  for (int bz = 0; bz < cz; bz++)
                    for (int by = 0; by < cy; by++) {
                      double *q = p + (bz ? oz : 0) + (by ? oy : 0);
                      q[0] = s;
                      if (cx == 2) q[ox] = s;
                    }
                }
              }
          }
    }
    /* exchange is the direction-keyed swap in recv_buf(); unpack-add
     * (gpu/v-26-messages/Faces.cc:554-669): every group on the subdomain
     * boundary sums its local copies and the received copies */
#pragma omp parallel for schedule(static)
    for (int gz = 0; gz <= G[2]; gz++)
      for (int gy = 0; gy <= G[1]; gy++)
        for (int gx = 0; gx <= G[0]; gx++) {
          const int onb = gx == 0 || gx == G[0] || gy == 0 || gy == G[1] || gz == 0 || gz == G[2];
          if (!onb) {
            gx = G[0] - 1; /* jump to the far face of this (gy,gz) row */
            continue;
          }
          if (gx % nm1 && gy % nm1 && gz % nm1) continue;
          const int gp[3] = {gx, gy, gz};
          gcop c;
          int nl;
          const int nc = v26_gather(o, ur, r, mb, gp, &c, &nl);
          if (nc < 2) continue;
          const double s = tree_sum(&c);
          for (int bz = 0; bz < c.cnt[2]; bz++)
            for (int by = 0; by < c.cnt[1]; by++)
              for (int bx = 0; bx < c.cnt[0]; bx++)
                if (c.p[bz][by][bx]) *c.p[bz][by][bx] = s;
        }
  }
}

void orc_v26_share(const orc_geom *g, double *u, int compute, int nsteps, int nthreads)
{
#ifdef _OPENMP
  const int saved = omp_get_max_threads();
  if (nthreads > 0) omp_set_num_threads(nthreads);
#else
  (void)nthreads;
#endif
  geo o;
  geo_make(g, &o);
  msgs mb;
  msgs_alloc(&o, &mb);
  for (int t = 0; t < nsteps; t++) v26_step(&o, u, compute, &mb);
  msgs_free(&mb);
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(saved);
#endif
}

/* ------------------------------------------------------------------ */
/* v-6: six face messages, three dimension sweeps                       */
/* (gpu/v-6-messages-basic/Faces.cc:65-173)                             */
/* ------------------------------------------------------------------ */

/* point (i, j) of dimension a lies on the subdomain boundary */
static inline int v6_on_boundary(const geo *o, int a, int i, int j)
{
  return (i == 0 && j == 0) || (i == o->n - 1 && j == o->m[a] - 1);
}

/* One share: sweeps in the reference's order z, y, x.  In the sweep of
 * dimension d every rank first packs its two face planes (the low face
 * i_d = 0 of element j_d = 0, the high face i_d = n-1 of element m_d-1;
 * Faces.cc:89-92,118-121,147-150), then adds to its low face the high face
 * its lower neighbour packed, sums each pair of neighbouring elements
 * (element j_d at n-1 with element j_d+1 at 0), and adds to its high face
 * the low face its upper neighbour packed (Faces.cc:105-113,134-142,
 * 163-171).  Faces carry the earlier sweeps' sums, so edges and corners
 * reach every copy: each point ends as the tree z pairs, y pairs, x pairs.
 * compute = 0 (the reference's v-6 ignores it) sums only points on the
 * subdomain boundary, as the other strategies do: a pair inside the
 * subdomain is taken only where its point lies on the boundary in another
 * dimension. */
static void v6_step(const geo *o, double *u, int compute, double *send)
{
  const int n = o->n;
  for (int d = 2; d >= 0; d--) {
    const int a = d == 0 ? 1 : 0, b = d == 2 ? 1 : 2;
    const long F = (long)n * n * o->m[a] * o->m[b];
    /* pack: face side s of rank r at send[(r*2 + s)*F + idx] */
#pragma omp parallel for schedule(static)
    for (int r = 0; r < o->nranks; r++)
      for (int jb = 0; jb < o->m[b]; jb++)
        for (int ja = 0; ja < o->m[a]; ja++)
          for (int ib = 0; ib < n; ib++)
            for (int ia = 0; ia < n; ia++) {
              const long idx = ia + (long)n * ib + (long)n * n * ja + (long)n * n * o->m[a] * jb;
              int i[3], j[3];
              i[a] = ia; i[b] = ib; j[a] = ja; j[b] = jb;
              i[d] = 0; j[d] = 0;
              send[((long)r * 2 + 0) * F + idx] = u[(long)r * o->R + gidx(o, i, j)];
              i[d] = n - 1; j[d] = o->m[d] - 1;
              send[((long)r * 2 + 1) * F + idx] = u[(long)r * o->R + gidx(o, i, j)];
            }
    /* updates */
#pragma omp parallel for schedule(static)
    for (int r = 0; r < o->nranks; r++) {
      int dm[3] = {0, 0, 0}, dp[3] = {0, 0, 0};
      dm[d] = -1;
      dp[d] = 1;
      const int lo = neighbor(o, r, dm), hi = neighbor(o, r, dp);
      double *ur = u + (long)r * o->R;
      for (int jb = 0; jb < o->m[b]; jb++)
        for (int ja = 0; ja < o->m[a]; ja++)
          for (int ib = 0; ib < n; ib++)
            for (int ia = 0; ia < n; ia++) {
              const long idx = ia + (long)n * ib + (long)n * n * ja + (long)n * n * o->m[a] * jb;
              const int keep = compute || v6_on_boundary(o, a, ia, ja) || v6_on_boundary(o, b, ib, jb);
              int i[3], j[3];
              i[a] = ia; i[b] = ib; j[a] = ja; j[b] = jb;
              if (lo >= 0) {
                i[d] = 0; j[d] = 0;
                double *p = ur + gidx(o, i, j);
                *p = *p + send[((long)lo * 2 + 1) * F + idx];
              }
              if (keep)
                for (int jd = 0; jd + 1 < o->m[d]; jd++) {
                  i[d] = n - 1; j[d] = jd;
                  double *p = ur + gidx(o, i, j);
                  i[d] = 0; j[d] = jd + 1;
                  double *q = ur + gidx(o, i, j);
                  const double s = *p + *q;
                  *p = s;
                  *q = s;
                }
              if (hi >= 0) {
                i[d] = n - 1; j[d] = o->m[d] - 1;
                double *p = ur + gidx(o, i, j);
                *p = *p + send[((long)hi * 2 + 0) * F + idx];
              }
            }
    }
  }
}

void orc_v6_share(const orc_geom *g, double *u, int compute, int nsteps)
{
  geo o;
  geo_make(g, &o);
  long fmax = 0;
  for (int d = 0; d < 3; d++) {
    const int a = d == 0 ? 1 : 0, b = d == 2 ? 1 : 2;
    const long F = (long)o.n * o.n * o.m[a] * o.m[b];
    if (F > fmax) fmax = F;
  }
  double *send = (double *)malloc(sizeof(double) * (size_t)(fmax * 2 * o.nranks));
  if (!send) return;
  for (int t = 0; t < nsteps; t++) v6_step(&o, u, compute, send);
  free(send);
}

/* ------------------------------------------------------------------ */
/* correctness check, gpu/main.cc:39-105                                 */
/* ------------------------------------------------------------------ */

double orc_compare(const orc_geom *g, const double *a, const double *b, int *npass,
                   int *where_rank, int where[6])
{
  geo o;
  geo_make(g, &o);
  const int n = o.n;
  double gmax = 0;
  int pass = 0;
  for (int r = 0; r < o.nranks; r++) {
    double mv = 0;
    int ml[6] = {0, 0, 0, 0, 0, 0};
    for (int jz = 0; jz < o.m[2]; jz++)
      for (int jy = 0; jy < o.m[1]; jy++)
        for (int jx = 0; jx < o.m[0]; jx++)
          for (int iz = 0; iz < n; iz++)
            for (int iy = 0; iy < n; iy++)
              for (int ix = 0; ix < n; ix++) {
                const int i[3] = {ix, iy, iz}, j[3] = {jx, jy, jz};
                const long k = (long)r * o.R + gidx(&o, i, j);
                const double ue = a[k], ve = b[k];
                const double denom = fabs(ue) + fabs(ve);
                const double d = (denom > 1e-15) ? fabs(ue - ve) / denom : 0;
                if (mv < d || d != d) {
                  mv = (d != d) ? INFINITY : d;
                  ml[0] = ix; ml[1] = iy; ml[2] = iz; ml[3] = jx; ml[4] = jy; ml[5] = jz;
                }
              }
    if (mv < 1e-15) pass++;
    if (r == 0 || mv > gmax) {
      gmax = mv;
      if (where_rank) *where_rank = r;
      if (where) memcpy(where, ml, sizeof(ml));
    }
  }
  if (npass) *npass = pass;
  return gmax;
}
