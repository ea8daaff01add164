/*
 * faces_oracle.h -- CPU oracle for the Faces halo-sum step.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the product path (the CUDA library,
 * the `faces` executable, the Python package) links, loads or calls this code.
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use it,
 * and only as the checker / the timed host baseline.
 *
 * Field layout (all functions): the reference's DArray<double,6> layout
 * (gpu/DArray.h:34-38,91-101) for one rank,
 *     idx = ix + n*iy + n^2*iz + n^3*jx + n^3*mx*jy + S4*jz,
 *     S4  = ceil(n^3*mx*my / 512) * 512          (page-padded jz stride),
 * and lx*ly*lz virtual ranks stored rank-major, rank r at offset r*S4*mz.
 * Rank r has coordinates kx = r % lx, ky = (r / lx) % ly, kz = r / (lx*ly)
 * (gpu/Mugs.cc:23-25).
 *
 * Three independent formulations of one share (one halo-sum step):
 *   orc_groups_share : global-mesh enumeration of every shared point; the sum
 *                      of its 2/4/8 copies is a tree in dimension order
 *                      (x pairs, then y pairs, then z pairs).
 *   orc_mugs_share   : restatement of the reference oracle Mugs::share
 *                      (gpu/Mugs.cc:86-416): in-place x, y, z pair passes per
 *                      rank, then 26 messages per rank added in the
 *                      reference's order.  periodic=0 is the reference;
 *                      periodic=1 generalises neighbor() with wrap-around and
 *                      direction-keyed message slots.
 *   orc_v26_share    : the v-26 strategy (gpu/v-26-messages/Faces.cc:111-678)
 *                      on the host with OpenMP: pack 26 raw boundary messages
 *                      per rank, inner sums of subdomain-interior groups,
 *                      direction-keyed buffer swap, unpack-add of
 *                      subdomain-boundary groups.  Sums use the same tree order
 *                      as orc_groups_share.  This is the timed CPU baseline.
 *
 * Exactness: on integer-valued inputs below 2^20 every formulation is exact
 * (sums of at most 8 integers; later steps scale by powers of two), so all
 * three agree bit for bit.  orc_groups_share and orc_v26_share agree bit for
 * bit on any input; orc_mugs_share agrees bit for bit with them on one
 * non-periodic rank on any input (its passes form the same tree).
 */
#pragma once
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_geom {
  int lx, ly, lz;   /* virtual rank grid */
  int mx, my, mz;   /* elements per rank */
  int n;            /* points per element edge (n >= 2) */
  int periodic;     /* 0: reference neighbours (MPI_PROC_NULL outside), 1: wrap */
} orc_geom;

/* 0 if the geometry is valid, else a negative code. */
int orc_check(const orc_geom *g);
/* jz stride S4 (doubles), doubles per rank S4*mz, total doubles. */
long orc_jz_stride(const orc_geom *g);
long orc_rank_doubles(const orc_geom *g);
long orc_total_doubles(const orc_geom *g);

/* gpu/main.cc:18 formula on every rank; padding left at zero. */
void orc_init_ref(const orc_geom *g, double *u);
/* integer-valued doubles uniform in [0,2^20): top 20 bits of
 * splitmix64(seed*0x9E3779B97F4A7C15 + linear index); padding zero. */
void orc_init_int(const orc_geom *g, double *u, uint64_t seed);
/* the integer init formula for one linear index (shared with the device) */
double orc_int_value(uint64_t seed, long index);

void orc_groups_share(const orc_geom *g, double *u, int compute, int nsteps);
void orc_mugs_share(const orc_geom *g, double *u, int compute, int nsteps);
/* nthreads <= 0: OpenMP default. */
void orc_v26_share(const orc_geom *g, double *u, int compute, int nsteps, int nthreads);
/* the v-6 strategy: z, y, x dimension sweeps of face messages and element
 * pairs (sums in the tree order z, y, x) */
void orc_v6_share(const orc_geom *g, double *u, int compute, int nsteps);

/* gpu/main.cc:39-105 check on every rank: max relative error
 * |a-b|/(|a|+|b|) (0 where the denominator is <= 1e-15) over the points of
 * all elements.  Returns the maximum over ranks; *npass = ranks whose maximum
 * is < 1e-15; *where (6 ints, may be NULL) = location of the global maximum. */
double orc_compare(const orc_geom *g, const double *a, const double *b, int *npass,
                   int *where_rank, int where[6]);

/* number of OpenMP threads the runtime will use */
int orc_max_threads(void);

#ifdef __cplusplus
}
#endif
