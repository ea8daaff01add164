// geom.cuh -- field geometry shared by the host API and the sm_103a kernels.
//
// A field is lx*ly*lz virtual ranks, each holding mx*my*mz spectral elements
// of n^3 FP64 points in the reference's DArray<double,6> layout
// (gpu/DArray.h:34-38,91-101):
//     idx = ix + n*iy + n^2*iz + n^3*jx + n^3*mx*jy + S4*jz,
//     S4  = ceil(n^3*mx*my/512)*512,
// ranks stored rank-major at stride S4*mz.  Rank r sits at
// (r % lx, (r/lx) % ly, r/(lx*ly)) (gpu/v-26-messages/Faces.cc:33-35).
//
// Neighbour directions are indexed dir = (dx+1) + 3*(dy+1) + 9*(dz+1); 13 is
// the rank itself, and the opposite of dir is 26-dir.  The message a rank
// sends toward direction d holds region(d): its points on the subdomain
// boundary facing d (for d_a = -1 the plane j_a = 0, i_a = 0; for d_a = +1 the
// plane j_a = m_a-1, i_a = n-1), listed with the free point indices fastest
// (x, y, z order) and then the free element indices -- the layout of the
// reference's zfs(ix,iy,jx,jy), yfs(ix,iz,jx,jz), xfs(iy,iz,jy,jz), xes(ix,jx)
// ... buffers (gpu/v-26-messages/Faces.cc:16-27).  Rank r receives from
// direction d what neighbour(r,d) sent toward -d: slots are keyed by
// direction, not by peer rank, so a periodic grid with l = 1 or 2 (where one
// peer is the neighbour in several directions) pairs the right faces.
#pragma once

#include <stdint.h>

#ifdef __CUDACC__
#define FACES_HD __host__ __device__ __forceinline__
#else
#define FACES_HD inline
#endif

namespace faces {

enum Mode : int {
  kDirect = 0,    // one owner per shared point across ranks; no messages
  kMessages = 1,  // v-26: pack 26 messages per rank, swap, unpack-add per rank
};

struct FieldDesc {
  double *u;          // all ranks
  long sjy, sjz, R;   // strides of jy, jz (doubles) and of a rank
  int n, m[3], L[3];  // n; mx,my,mz; lx,ly,lz
  int periodic;
  int mode;
  int nranks;
  // messages (mode kMessages): send buffers of all ranks; off[r*27+dir] is
  // the offset of rank r's buffer toward dir (-1: no neighbour there)
  double *msg;
  const long *msg_off;
  // recv_off[r*27+dir]: offset in msg of what rank r receives from
  // direction dir -- neighbour(r,dir)'s buffer toward -dir -- or -1
  const long *recv_off;
  // nbr[r*27+dir]: neighbour rank in direction dir, -1 outside a
  // non-periodic grid (MPI_PROC_NULL in gpu/v-26-messages/Faces.cc:92-103)
  const int *nbr;
};

FACES_HD int dir_index(int dx, int dy, int dz) { return (dx + 1) + 3 * (dy + 1) + 9 * (dz + 1); }

FACES_HD long jz_stride(int n, int mx, int my)
{
  const long page = 512;  // 4096-byte DArray page padding
  const long s = (long)n * n * n * mx * my;
  return ((s - 1) / page + 1) * page;
}

FACES_HD long elem_index(const FieldDesc &f, int ix, int iy, int iz, int jx, int jy, int jz)
{
  const long n = f.n;
  return ix + n * iy + n * n * iz + n * n * n * jx + f.sjy * jy + f.sjz * jz;
}

// position inside region(d)'s message of a point whose free coordinates are
// (i[a], j[a]) for every a with d[a] == 0
FACES_HD long region_pos(const FieldDesc &f, const int d[3], const int i[3], const int j[3])
{
  long pos = 0, mul = 1;
  for (int a = 0; a < 3; a++)
    if (d[a] == 0) { pos += i[a] * mul; mul *= f.n; }
  for (int a = 0; a < 3; a++)
    if (d[a] == 0) { pos += j[a] * mul; mul *= f.m[a]; }
  return pos;
}

FACES_HD long region_size(const FieldDesc &f, const int d[3])
{
  long s = 1;
  for (int a = 0; a < 3; a++)
    if (d[a] == 0) s *= (long)f.n * f.m[a];
  return s;
}

}  // namespace faces
