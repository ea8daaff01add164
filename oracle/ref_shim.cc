// ref_shim.cc -- C entry point around the reference's own Mugs oracle
// (gpu/Mugs.cc, compiled unmodified from the reference tree by
// oracle/Makefile's `ref` target).  Test infrastructure only: it checks this
// project's restatement in oracle/faces_oracle.c.
//
// mugs_ref_share(): u holds lx*ly*lz ranks in the padded DArray layout
// (gpu/DArray.h:91-101), rank-major.  Each rank runs on its own thread of the
// single-process MPI stand-in; it copies its part into the reference's host
// Array<double,6> (gpu/Array.h), runs Mugs::share nsteps times
// (gpu/main.cc:166-167) and copies the result back.
#include <omp.h>

#include <cstdio>
#include <iostream>
#include <sstream>

#include "mpi.h"
#include "Mugs.h"

namespace {

struct Job {
  int lx, ly, lz, mx, my, mz, n, compute, nsteps, nthreads;
  double *u;
  long jz_stride, rank_stride;
};

void run_rank(int rank, void *arg)
{
  Job &j = *static_cast<Job *>(arg);
  omp_set_num_threads(j.nthreads);
  const int n = j.n;
  Array<double, 6> v(n, n, n, j.mx, j.my, j.mz);
  double *ur = j.u + rank * j.rank_stride;
  const long plane = (long)n * n * n * j.mx * j.my;
  for (int jz = 0; jz < j.mz; jz++)
    for (long p = 0; p < plane; p++) v[jz * plane + p] = ur[jz * j.jz_stride + p];
  {
    // the constructor prints an "Initialized Mugs" line on rank 0
    std::stringstream sink;
    std::streambuf *old = std::cout.rdbuf(sink.rdbuf());
    Mugs mugs(rank, j.lx, j.ly, j.lz, j.mx, j.my, j.mz, n);
    std::cout.rdbuf(old);
    for (int s = 0; s < j.nsteps; s++) mugs.share(v, j.compute != 0);
  }
  for (int jz = 0; jz < j.mz; jz++)
    for (long p = 0; p < plane; p++) ur[jz * j.jz_stride + p] = v[jz * plane + p];
}

}  // namespace

extern "C" int mugs_ref_share(int lx, int ly, int lz, int mx, int my, int mz, int n, int compute,
                              int nsteps, double *u, int nthreads)
{
  if (n < 2 || lx < 1 || ly < 1 || lz < 1 || mx < 1 || my < 1 || mz < 1) return -1;
  Job j{lx, ly, lz, mx, my, mz, n, compute, nsteps, nthreads > 0 ? nthreads : 1, u, 0, 0};
  const long page = 512;
  const long plane = (long)n * n * n * mx * my;
  j.jz_stride = ((plane - 1) / page + 1) * page;
  j.rank_stride = j.jz_stride * mz;
  mpistub_run(lx * ly * lz, run_rank, &j);
  return 0;
}
